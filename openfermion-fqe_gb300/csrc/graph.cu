// K1: string graph of a sector, built on the device.
//
// Reference: FciGraph (fci_graph.py:108-154) with the natives
// lexicographic_bitstring_generator (lib/bitstring.c:29-45), calculate_Z_matrix
// (lib/fci_graph.c:27-54), calculate_string_address (:136-147),
// build_mapping_strings (:76-121) and map_to_deexc (fci_graph.py:36-63).
//
// Tables per spin:
//   strings[len]        bit masks at their Knowles-Handy address
//   zmat[nele][norb]    addressing matrix
//   dexc[len][ndexc][3] per target: (source, i*norb+j, sign), ij ascending —
//                       the order map_to_deexc produces, since each target
//                       appears at most once in every (i, j) map
//   tab_full[ij][len]   per pair and target: 0 or sign*(source+1)
//   tab_tri[p][len]     same on compressed pairs p = tri(max, min); at most one
//                       of E_ij, E_ji reaches a given target, so one entry
//                       suffices
#include <cstdlib>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace fqegpu {

__device__ __forceinline__ int64_t dbinom(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  if (k > n - k) k = n - k;
  int64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

// Z[k-1][l-1] for k < nele: sum_{m=norb-l+1}^{norb-k} C(m, nele-k) - C(m-1, nele-k-1)
// Z[nele-1][l-1] = l - nele.  Entries outside the reference's loops stay 0.
__global__ void k_zmatrix(int norb, int nele, int32_t* __restrict__ Z) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nele * norb) return;
  const int k = id / norb + 1, l = id % norb + 1;
  int32_t v = 0;
  if (k < nele) {
    if (l >= k && l <= norb - nele + k) {
      int64_t acc = 0;
      for (int m = norb - l + 1; m <= norb - k; ++m)
        acc += dbinom(m, nele - k) - dbinom(m - 1, nele - k - 1);
      v = (int32_t)acc;
    }
  } else {
    if (l >= nele) v = l - nele;
  }
  Z[id] = v;
}

__device__ __forceinline__ int str_index(uint64_t s, const int32_t* __restrict__ Z,
                                         int norb) {
  int idx = 0, k = 0;
  while (s) {
    const int p = __ffsll((long long)s) - 1;
    idx += Z[k * norb + p];
    ++k;
    s &= s - 1;
  }
  return idx;
}

// One thread per rank r of the colex (= increasing integer) order of
// nele-subsets: unrank by the combinatorial number system, then place the
// string at its address.
__global__ void k_strings(int norb, int nele, int64_t len,
                          const int32_t* __restrict__ Z,
                          uint64_t* __restrict__ out) {
  const int64_t r0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r0 >= len) return;
  if (nele == 0) {
    out[0] = 0ull;
    return;
  }
  int64_t r = r0;
  uint64_t s = 0;
  int c = norb - 1;
  for (int k = nele; k >= 1; --k) {
    while (dbinom(c, k) > r) --c;
    s |= 1ull << c;
    r -= dbinom(c, k);
    --c;
  }
  out[str_index(s, Z, norb)] = s;
}

__device__ __forceinline__ int sign_between(uint64_t s, int i, int j) {
  const int lo = min(i, j), hi = max(i, j);
  if (hi - lo < 2) return 1;
  const uint64_t mask = ((1ull << hi) - 1) & ~((2ull << lo) - 1);
  return (__popcll(s & mask) & 1) ? -1 : 1;
}

// One thread per target string T: enumerate E_ij with i in T and j == i or
// j not in T, i-major then j ascending; source S = T - i + j.
__global__ void k_dexc(int norb, int64_t len, int ndexc,
                       const uint64_t* __restrict__ strings,
                       const int32_t* __restrict__ Z,
                       int32_t* __restrict__ dexc,
                       int32_t* __restrict__ tab_full,
                       int32_t* __restrict__ tab_tri) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= len) return;
  const uint64_t T = strings[t];
  int32_t* d = dexc + 3 * t * ndexc;
  int k = 0;
  for (int i = 0; i < norb; ++i) {
    if (!(T >> i & 1ull)) continue;
    for (int j = 0; j < norb; ++j) {
      int src, sg;
      if (j == i) {
        src = (int)t;
        sg = 1;
      } else if (!(T >> j & 1ull)) {
        const uint64_t S = (T & ~(1ull << i)) | (1ull << j);
        src = str_index(S, Z, norb);
        sg = sign_between(T, i, j);
      } else {
        continue;
      }
      if (k < ndexc) {
        d[3 * k + 0] = src;
        d[3 * k + 1] = i * norb + j;
        d[3 * k + 2] = sg;
      }
      ++k;
      const int32_t code = sg * (src + 1);
      tab_full[(int64_t)(i * norb + j) * len + t] = code;
      tab_tri[(int64_t)tri_index(i, j) * len + t] = code;
    }
  }
}

// Reference-format maps, one CTA per (i, j): entries (source, target, sign)
// over sources in address order; the position of each entry is a block-wide
// running count of the predicate.
__global__ void k_maps(int norb, int64_t len, const uint64_t* __restrict__ strings,
                       const int32_t* __restrict__ Z,
                       const int64_t* __restrict__ offsets,
                       int32_t* __restrict__ maps) {
  const int ij = blockIdx.x;
  const int i = ij / norb, j = ij % norb;
  __shared__ int warp_counts[32];
  __shared__ int64_t base;
  if (threadIdx.x == 0) base = offsets[ij];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int64_t s0 = 0; s0 < len; s0 += blockDim.x) {
    const int64_t s = s0 + threadIdx.x;
    bool hit = false;
    uint64_t S = 0;
    if (s < len) {
      S = strings[s];
      hit = (i == j) ? ((S >> i & 1ull) != 0)
                     : ((S >> j & 1ull) && !(S >> i & 1ull));
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) warp_counts[warp] = __popc(ballot);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < nwarps; ++w) {
      if (w < warp) before += warp_counts[w];
      total += warp_counts[w];
    }
    before += __popc(ballot & ((1u << lane) - 1u));
    if (hit) {
      int32_t* m = maps + 3 * (base + before);
      if (i == j) {
        m[0] = (int32_t)s; m[1] = (int32_t)s; m[2] = 1;
      } else {
        const uint64_t T = (S & ~(1ull << j)) | (1ull << i);
        m[0] = (int32_t)s;
        m[1] = str_index(T, Z, norb);
        m[2] = sign_between(S, i, j);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base += total;
    __syncthreads();
  }
}

static void free_spin(SpinTables& t) {
  cudaFree(t.strings);
  cudaFree(t.zmat);
  cudaFree(t.dexc);
  cudaFree(t.tab_full);
  cudaFree(t.tab_tri);
  t = SpinTables();
}

static int build_spin(int norb, int nele, cudaStream_t st, SpinTables& t) {
  t.nele = nele;
  t.len = binom_host(norb, nele);
  t.ndexc = nele * (norb - nele + 1);
  const int64_t len = t.len;
  const int P = norb * norb, PT = norb * (norb + 1) / 2;
  FQE_CUDA(dev_alloc(&t.strings, sizeof(uint64_t) * len));
  FQE_CUDA(dev_alloc(&t.zmat, sizeof(int32_t) * (size_t)(nele * norb > 0 ? nele * norb : 1)));
  FQE_CUDA(dev_alloc(&t.dexc, sizeof(int32_t) * 3 * (size_t)(len * t.ndexc > 0 ? len * t.ndexc : 1)));
  FQE_CUDA(dev_alloc(&t.tab_full, sizeof(int32_t) * (size_t)(P > 0 ? P : 1) * len));
  FQE_CUDA(dev_alloc(&t.tab_tri, sizeof(int32_t) * (size_t)(PT > 0 ? PT : 1) * len));
  FQE_CUDA(cudaMemsetAsync(t.tab_full, 0, sizeof(int32_t) * (size_t)(P > 0 ? P : 1) * len, st));
  FQE_CUDA(cudaMemsetAsync(t.tab_tri, 0, sizeof(int32_t) * (size_t)(PT > 0 ? PT : 1) * len, st));
  if (nele * norb > 0) {
    k_zmatrix<<<(nele * norb + 127) / 128, 128, 0, st>>>(norb, nele, t.zmat);
    FQE_CUDA(cudaGetLastError());
  }
  k_strings<<<(unsigned)((len + 255) / 256), 256, 0, st>>>(norb, nele, len, t.zmat,
                                                           t.strings);
  FQE_CUDA(cudaGetLastError());
  if (t.ndexc > 0) {
    k_dexc<<<(unsigned)((len + 127) / 128), 128, 0, st>>>(
        norb, len, t.ndexc, t.strings, t.zmat, t.dexc, t.tab_full, t.tab_tri);
    FQE_CUDA(cudaGetLastError());
  }
  return FQEGPU_OK;
}

}  // namespace fqegpu

using namespace fqegpu;

extern "C" int fqegpu_graph_create(int norb, int nalpha, int nbeta, void* stream,
                                   fqegpu_graph* out) {
  clear_error();
  FQE_CHECK_ARG(out != nullptr, "out is NULL");
  FQE_CHECK_ARG(norb >= 0 && norb <= 63, "norb must be in [0, 63]");
  FQE_CHECK_ARG(nalpha >= 0 && nalpha <= norb, "nalpha must be in [0, norb]");
  FQE_CHECK_ARG(nbeta >= 0 && nbeta <= norb, "nbeta must be in [0, norb]");
  FQE_CHECK_ARG(binom_host(norb, nalpha) < (1ll << 31) &&
                    binom_host(norb, nbeta) < (1ll << 31),
                "string space too large for 32-bit addresses");
  cudaStream_t st = (cudaStream_t)stream;
  auto* g = new (std::nothrow) fqegpu_graph_s();
  if (!g) {
    set_error("host allocation failed");
    return FQEGPU_ERR_NOMEM;
  }
  g->norb = norb;
  g->nalpha = nalpha;
  g->nbeta = nbeta;
  int s = build_spin(norb, nalpha, st, g->a);
  if (s == FQEGPU_OK) s = build_spin(norb, nbeta, st, g->b);
  if (s == FQEGPU_OK) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_error("graph build: %s", cudaGetErrorString(e));
      s = FQEGPU_ERR_CUDA;
    }
  }
  if (s != FQEGPU_OK) {
    free_spin(g->a);
    free_spin(g->b);
    delete g;
    return s;
  }
  *out = g;
  return FQEGPU_OK;
}

extern "C" int fqegpu_graph_destroy(fqegpu_graph g) {
  if (!g) return FQEGPU_OK;
  free_spin(g->a);
  free_spin(g->b);
  delete g;
  return FQEGPU_OK;
}

extern "C" int fqegpu_graph_dims(fqegpu_graph g, int64_t* lena, int64_t* lenb,
                                 int* ndexca, int* ndexcb) {
  clear_error();
  FQE_CHECK_ARG(g != nullptr, "graph is NULL");
  if (lena) *lena = g->a.len;
  if (lenb) *lenb = g->b.len;
  if (ndexca) *ndexca = g->a.ndexc;
  if (ndexcb) *ndexcb = g->b.ndexc;
  return FQEGPU_OK;
}

static const SpinTables* spin_of(fqegpu_graph g, int spin) {
  return spin == 0 ? &g->a : &g->b;
}

extern "C" int fqegpu_graph_strings(fqegpu_graph g, int spin, uint64_t* h_out) {
  clear_error();
  FQE_CHECK_ARG(g && h_out && (spin == 0 || spin == 1), "bad arguments");
  const SpinTables* t = spin_of(g, spin);
  FQE_CUDA(cudaMemcpy(h_out, t->strings, sizeof(uint64_t) * t->len,
                      cudaMemcpyDeviceToHost));
  return FQEGPU_OK;
}

extern "C" int fqegpu_graph_zmatrix(fqegpu_graph g, int spin, int32_t* h_out) {
  clear_error();
  FQE_CHECK_ARG(g && h_out && (spin == 0 || spin == 1), "bad arguments");
  const SpinTables* t = spin_of(g, spin);
  if (t->nele * g->norb == 0) return FQEGPU_OK;
  FQE_CUDA(cudaMemcpy(h_out, t->zmat, sizeof(int32_t) * t->nele * g->norb,
                      cudaMemcpyDeviceToHost));
  return FQEGPU_OK;
}

extern "C" int fqegpu_graph_dexc(fqegpu_graph g, int spin, int32_t* h_out) {
  clear_error();
  FQE_CHECK_ARG(g && h_out && (spin == 0 || spin == 1), "bad arguments");
  const SpinTables* t = spin_of(g, spin);
  if (t->ndexc == 0) return FQEGPU_OK;
  FQE_CUDA(cudaMemcpy(h_out, t->dexc, sizeof(int32_t) * 3 * t->len * t->ndexc,
                      cudaMemcpyDeviceToHost));
  return FQEGPU_OK;
}

// Map (i, j) holds C(norb-1, nele-1) entries when i == j and C(norb-2, nele-1)
// otherwise (strings with j occupied and i empty).
static void map_lengths(int norb, int nele, std::vector<int32_t>& out) {
  out.assign((size_t)norb * norb, 0);
  for (int i = 0; i < norb; ++i)
    for (int j = 0; j < norb; ++j)
      out[(size_t)i * norb + j] =
          (int32_t)(i == j ? binom_host(norb - 1, nele - 1)
                           : binom_host(norb - 2, nele - 1));
}

extern "C" int fqegpu_graph_map_lengths(fqegpu_graph g, int spin, int32_t* h_out) {
  clear_error();
  FQE_CHECK_ARG(g && h_out && (spin == 0 || spin == 1), "bad arguments");
  std::vector<int32_t> l;
  map_lengths(g->norb, spin_of(g, spin)->nele, l);
  if (!l.empty()) memcpy(h_out, l.data(), sizeof(int32_t) * l.size());
  return FQEGPU_OK;
}

extern "C" int fqegpu_graph_maps(fqegpu_graph g, int spin, int32_t* h_out) {
  clear_error();
  FQE_CHECK_ARG(g && h_out && (spin == 0 || spin == 1), "bad arguments");
  const SpinTables* t = spin_of(g, spin);
  const int norb = g->norb;
  if (norb == 0) return FQEGPU_OK;
  std::vector<int32_t> l;
  map_lengths(norb, t->nele, l);
  std::vector<int64_t> off((size_t)norb * norb + 1, 0);
  for (size_t k = 0; k < l.size(); ++k) off[k + 1] = off[k] + l[k];
  const int64_t total = off.back();
  if (total == 0) return FQEGPU_OK;
  int64_t* d_off = nullptr;
  int32_t* d_maps = nullptr;
  FQE_CUDA(dev_alloc(&d_off, sizeof(int64_t) * off.size()));
  cudaError_t e = dev_alloc(&d_maps, sizeof(int32_t) * 3 * total);
  if (e == cudaSuccess)
    e = cudaMemcpy(d_off, off.data(), sizeof(int64_t) * off.size(),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_maps<<<norb * norb, 256>>>(norb, t->len, t->strings, t->zmat, d_off, d_maps);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpy(h_out, d_maps, sizeof(int32_t) * 3 * total,
                   cudaMemcpyDeviceToHost);
  cudaFree(d_off);
  cudaFree(d_maps);
  if (e != cudaSuccess) {
    set_error("graph maps: %s", cudaGetErrorString(e));
    return FQEGPU_ERR_CUDA;
  }
  return FQEGPU_OK;
}

namespace fqegpu {
// Builds the tables of one spin into caller-provided device memory (`mem`,
// `bytes`) with the same kernels as fqegpu_graph_create; returns the number
// of bytes used, or -1 when they do not fit.
int64_t build_spin_into(int norb, int nele, void* mem, size_t bytes, cudaStream_t st,
                        SpinTables& t) {
  t.nele = nele;
  t.len = binom_host(norb, nele);
  t.ndexc = nele * (norb - nele + 1);
  const int64_t len = t.len;
  const int P = norb * norb, PT = norb * (norb + 1) / 2;
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t s_str = up(sizeof(uint64_t) * len);
  const size_t s_z = up(sizeof(int32_t) * (size_t)(nele * norb > 0 ? nele * norb : 1));
  const size_t s_dexc = up(sizeof(int32_t) * 3 * (size_t)(len * t.ndexc > 0 ? len * t.ndexc : 1));
  const size_t s_full = up(sizeof(int32_t) * (size_t)(P > 0 ? P : 1) * len);
  const size_t s_tri = up(sizeof(int32_t) * (size_t)(PT > 0 ? PT : 1) * len);
  const size_t need = s_str + s_z + s_dexc + s_full + s_tri;
  if (need > bytes) return -1;
  unsigned char* p = static_cast<unsigned char*>(mem);
  t.strings = reinterpret_cast<uint64_t*>(p);
  t.zmat = reinterpret_cast<int32_t*>(p + s_str);
  t.dexc = reinterpret_cast<int32_t*>(p + s_str + s_z);
  t.tab_full = reinterpret_cast<int32_t*>(p + s_str + s_z + s_dexc);
  t.tab_tri = reinterpret_cast<int32_t*>(p + s_str + s_z + s_dexc + s_full);
  if (cudaMemsetAsync(t.tab_full, 0, s_full + s_tri, st) != cudaSuccess) return -1;
  if (nele * norb > 0) k_zmatrix<<<(nele * norb + 127) / 128, 128, 0, st>>>(norb, nele, t.zmat);
  k_strings<<<(unsigned)((len + 255) / 256), 256, 0, st>>>(norb, nele, len, t.zmat, t.strings);
  if (t.ndexc > 0)
    k_dexc<<<(unsigned)((len + 127) / 128), 128, 0, st>>>(norb, len, t.ndexc, t.strings, t.zmat,
                                                          t.dexc, t.tab_full, t.tab_tri);
  if (cudaGetLastError() != cudaSuccess) return -1;
  return (int64_t)need;
}
}  // namespace fqegpu
