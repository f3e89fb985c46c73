// Tensor-core pair contraction with Ozaki splitting (FQEGPU_PREC_OZAKI).
//
// G[p][I] = sum_q V[p][q] D[q][I] with V the real pair matrix (fqe_data.py
// :658-681 compressed form, one-body part folded in) and D[q][I] = <I|E_q|psi>.
// GB300's FP64 pipe runs at ~1.1 TFLOP/s, so the FP64 operands are split into
// BF16 slices and contracted on the 5th-generation tensor cores:
//
//   V[p][q] = 2^{eV(p)}   sum_{a=1..5} v_a[p][q] 2^{-8a},  v_a in {-255..255}
//   D[q][I] = 2^{g0 + 1}  sum_{b=1..6} d_b[q][I] 2^{-8b},  d_b in {-256..256}
//
// V: sign-magnitude bytes of the 40-bit fixed-point rows (row exponent eV(p)).
// D: psi is scaled by ONE global exponent g0 (max |Re|, |Im| of psi < 2^g0)
// to a 47-bit fixed-point integer and cut once per apply into six balanced
// base-256 digits in [-128, 128] (k_oz_digits).  Every D entry is the sum of
// at most two psi entries with signs +-1 (one alpha source, one beta source:
// every target string has at most one source under each pair operator), so
// D's digit b is the signed sum of its sources' digits b, in [-256, 256]:
// exact in BF16.  The producers therefore only gather digits and add them (no
// rounding, no per-determinant exponent).  Slices are stored as their true
// values (digit * 2^{-8b}), so every product lands on one absolute scale and
// the products are grouped by level L = a + b into four TMEM accumulators:
// L = 2, 3 and 4 sum integers times 2^{-8L} that stay below 2^24 (exact in
// FP32; level 4 can only exceed it for near-saturated digits); L = 5..7
// share one accumulator whose FP32 rounding sits ~2^-48 below level 2.
// Levels >= 8 are dropped: 20 BF16 products per tile (a <= 5, b <= 6).  The
// four accumulators are combined by a chain of exact two-sums into an FP32
// pair (h, l) (h the rounded sum, l the summed rounding errors: ~48 bits; no
// level is assumed to hold the leading bits, since at one global scale a
// small column starts in level 4 or later), left unnormalised for the
// scatter's FP32-pair sum, and scaled by 2^{eV(p) + g0 + 1}.  Modelled error on sigma (numpy model,
// tests/test_ozaki_model.py): ~1e-12 for a spread-out psi, 2-3e-12 for one
// concentrated on a few determinants, ~5e-13 for the high-order terms of a
// Taylor series, against 1.7-4.6e-12 for exact per-determinant exponents.
//
// Kernels:
//   k_oz_rowexp, k_oz_globalexp  g0 (and a flag for Inf/NaN input).
//   k_oz_digits  the six digit planes of psi: [N] 16-byte words (digits 1-4,
//               each a bf16x2 of the real and imaginary digit) and [N] 8-byte
//               words (digits 5-6).
//   k_oz_fused  persistent, one CTA per SM: eight producer warps gather the
//               sources' digits through the per-pair target tables (table
//               entries loaded one K chunk ahead), add them with their signs
//               (bf16x2, exact) and write the six D slices of a K chunk of a
//               tile pair (64 determinants) straight into a shared-memory
//               ring in the tensor core's canonical K-major image, one
//               bank-conflict-free 16-byte row per lane and slice; the MMA
//               warp issues 128 x NP x 16 tcgen05.mma (A = the D chunk, B = V
//               slices resident in shared memory); eight epilogue warps drain
//               the four TMEM accumulators (loads of the next four columns in
//               flight while the current four are combined), release them
//               before their last stores, and store G coalesced as FP32 pairs
//               [P][lena][w].  No D image passes through HBM.
//   k_oz_scatter  sigma from G in FP32-pair arithmetic.
// Every wait in k_oz_fused is bounded; on a timeout the kernel records an
// error, lets the other roles leave and frees its TMEM (its only
// asynchronous operations are MMAs, which it waits for).
#include <cuda_bf16.h>
#include <math_constants.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ham.cuh"
#include "tcgen05.cuh"

namespace fqegpu {

namespace {
constexpr int kSlices = 5;     // slices of V
constexpr int kDSlices = 6;    // slices (digits) of D
constexpr int kMaxLevel = 7;   // pairs (a, b) with a + b <= 7 are contracted
constexpr int kM = 128;        // MMA M (pairs, padded)
constexpr int kN = 64;         // real columns of one slice tile
constexpr int kNM = 128;       // MMA N: two slice tiles
constexpr int kDets = 32;      // determinants per slice tile
constexpr int kSuperTiles = 32;  // default tiles per column super-block (1024 columns)
constexpr int kChunkK = 16;    // K columns per streamed slice chunk (one MMA k-step)
constexpr int kChunkElems = kN * kChunkK;  // 1024 BF16 = 2 KB
constexpr int kPairChunkElems = 2 * kChunkElems;  // a K chunk of both tiles of a pair: 4 KB
constexpr int kSlotBytes = kDSlices * kPairChunkElems * 2;  // one K chunk, six slices: 24 KB
constexpr int kMaxRing = 16;   // ring depth (bounded by shared memory)
constexpr int kEpiWarps = 8;   // two per TMEM lane quarter, NP / 2 columns each
constexpr int kMmaWarp = 8;
constexpr int kProdWarp0 = 9;   // producer warps 9 .. 16
constexpr int kProdWarps = 8;   // 256 threads: (64 determinants) x (4 quarters of a chunk)
constexpr int kThreads = (kProdWarp0 + kProdWarps) * 32;  // 17 warps
constexpr int kRegWarps = 20;  // register budget of the launch bounds
constexpr int kAccs = 4;           // levels 2, 3, 4 and 5..7
constexpr uint32_t kTmemCols = kAccs * kNM;  // 512: one accumulator set
constexpr long long kWaitCycles = 4000000000ll;  // default wait limit: ~2 s at 2 GHz
constexpr int kExpZero = -2000;
constexpr int kExpNonFinite = 30000;  // row exponent of a row holding Inf or NaN
}  // namespace

struct OzakiPlan {
  int P = 0, KP = 0;
  int npass = 1, NP = 0;               // output pairs in passes of NP rows
  int64_t wb = 0;                      // beta columns per block (multiple of 32)
  __nv_bfloat16* d_vslices = nullptr;  // [npass][5][NP * KP] canonical K-major
  int32_t* d_vexp = nullptr;           // [npass * NP] row exponents
  uint4* d_pdA = nullptr;              // [N] digits 1-4 of psi (bf16x2 re, im each)
  uint2* d_pdB = nullptr;              // [N] digits 5-6
  int32_t* d_rowexp = nullptr;         // [lena]
  int32_t* d_misc = nullptr;           // [0] = global exponent, [1] = error
  float4* d_G = nullptr;               // [P][lena][wb]
  int32_t* d_tabTA = nullptr;          // [lena][KP] target tables, pair index fastest
  int32_t* d_tabTB = nullptr;          // [lenb][KP]
  // beta-column blocks only: per block and target column, the pairs whose
  // beta source lies in the block, CSR: offsets [nblk][lenb + 1], entries
  // (pair, sign * (source - c0 + 1))
  int32_t* d_boff = nullptr;
  int2* d_bent = nullptr;
  int ring = 0;
  int nsm = 0;
  size_t smem = 0;
  // error reporting without a host synchronisation per apply: d_misc[1] is
  // a sticky error word (set by a kernel whose bounded wait gave up, cleared
  // only by a check); after each apply it is copied to pinned h_err and
  // err_ev recorded, so the next apply can poll it without blocking
  int32_t* h_err = nullptr;
  cudaEvent_t err_ev = nullptr;
  bool err_pending = false;
  // bounded-wait limit (clock cycles) and a test-only fault injection: when
  // skip_slot >= 0 the producers of CTA 0 leave that ring slot of its first
  // tile pair unfilled, so the MMA warp's wait on it must run out
  long long wait_cycles = kWaitCycles;
  int skip_slot = -1;
  // tuning (fqegpu_ham_set_tuning): tiles per column super-block, and
  // whether this operator runs the FP64 kernels (chosen by an autotuner for
  // small sectors, where the tensor-core form's fixed costs dominate)
  int super = kSuperTiles;
  bool use_fp64 = false;
};

struct OzArgs {
  int P, KP, ring;
  int NP, p0;        // this pass: N = NP output pairs starting at p0
  int64_t lena, lenb, ntiles;  // ntiles: tiles of this beta-column block
  int nb;            // tiles per alpha row in this block
  int64_t c0, gld;   // first column of the block; row length of G (block width)
  int super;         // tiles per column super-block of the tile order
  const int32_t* tabA;
  const int32_t* tabB;
  const int32_t* tabTA;  // [lena][KP]: the 8 pairs of an octet are 32 contiguous bytes
  const int32_t* tabTB;  // [lenb][KP]
  const uint4* pdA;  // digit planes of psi (k_oz_digits)
  const uint2* pdB;
  const int32_t* misc;
  const __nv_bfloat16* vslices;
  const int32_t* vexp;
  float4* G;
  int32_t* err;
  long long wait_cycles;  // limit of every bounded wait
  int skip_slot;          // test-only: slot of CTA 0's first tile pair left unfilled (-1: none)
};

// Tile t -> (alpha row, first beta column).  Tiles are visited in column
// super-blocks of A.super tiles (1024 determinants of a row), alpha rows
// within a super-block: the 16-byte psi segments the alpha-source gathers read
// (one 1024-column slice of every row, 16 KB each) then stay L2-resident.
__device__ __forceinline__ void tile_coords(const OzArgs& A, int64_t t, int64_t& ia,
                                            int64_t& ib0) {
  const int64_t per_super = A.lena * A.super;
  const int64_t sb = t / per_super;
  const int64_t r = t - sb * per_super;
  const int64_t w = min((int64_t)A.super, (int64_t)A.nb - sb * A.super);
  ia = r / w;
  ib0 = A.c0 + (sb * A.super + (r - ia * w)) * kDets;
}

// Bounded wait that also gives up when another role has aborted.
__device__ __forceinline__ bool oz_wait(uint64_t* bar, uint32_t parity,
                                        volatile int* abort_flag, long long limit) {
  if (tc::mbar_try_wait(bar, parity)) return true;  // fast path: no clock read
  const long long t0 = clock64();
  for (uint32_t it = 0;; ++it) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u) {
      if (*abort_flag) return false;
      if (clock64() - t0 > limit) return false;
    }
  }
}

// Bounded wait that ignores the abort flag: for copies already issued, which
// complete on their own (they depend on nothing but global memory).
__device__ __forceinline__ bool oz_wait_drain(uint64_t* bar, uint32_t parity, long long limit) {
  const long long t0 = clock64();
  for (uint32_t it = 0;; ++it) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u && clock64() - t0 > limit) return false;
  }
}

__device__ __forceinline__ void oz_abort(volatile int* abort_flag, int32_t* err, int code) {
  *abort_flag = 1;
  atomicExch(err, code);
}

// s + e = a + b exactly (Knuth's two-sum, FP32).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Accumulator of the product of V slice a and D digit b: levels 2, 3, 4 and
// 5..7.
__host__ __device__ constexpr int acc_of(int a, int b) { return a + b <= 4 ? a + b - 2 : 3; }

// 2^e as a float for -126 <= e <= 127.
__device__ __forceinline__ float pow2f(int e) {
  return __int_as_float((e + 127) << 23);
}

// x * 2^e in two exact steps (covers |e| <= 252; below that the result is
// under FP32's range and flushes to zero).
__device__ __forceinline__ float scale2(float x, int e) {
  if (e < -252) return 0.0f;
  e = min(e, 254);
  const int e1 = e / 2, e2 = e - e1;
  return (x * pow2f(e1)) * pow2f(e2);
}

// The digit planes of psi[src]: word k < 4 of `a` or word k - 4 of `b`
// holds digit k + 1 as a bf16x2 (real, imaginary).
__device__ __forceinline__ uint32_t digit_word(const uint4& a, const uint2& b, int k) {
  return k == 0 ? a.x : k == 1 ? a.y : k == 2 ? a.z : k == 3 ? a.w : k == 4 ? b.x : b.y;
}

// ---- the fused contraction: gather + digit slices + tcgen05 MMAs + epilogue --
// One MMA tile is a pair of slice tiles: 64 determinants = 128 real rows.  The
// MMA is G^T = D^T V^T: A = a 128-row K chunk (16 pairs) of D slice b, B = V
// slice a (NP rows = output pairs, resident in shared memory), D in TMEM = 128
// lanes (determinant, real/imaginary) x NP columns per level accumulator
// (4 x NP <= 512 columns, single-buffered); with lanes = determinants the
// epilogue's G stores are coalesced (a warp writes 16 determinants x 16 B of
// one pair).
// Persistent, one CTA per SM, 17 warps (registers are granted to warps in
// fours, so 17 warps at 96 registers fit where 21 did not):
//   warps 0-7   epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (16
//               determinants of one slice tile), columns = the pairs of half
//               w / 4; combines the four level sums, scales and stores G four
//               columns at a time, then releases the accumulators;
//   warp 8      TMEM allocation and the MMA issue loop (lane 0 issues);
//   warps 9-16  producers: one thread per (determinant of the tile pair,
//               quarter of the K chunk = 4 pairs).  For each K chunk they
//               read the target tables of their four pairs, gather the digit
//               words of each pair's (at most two) sources, add them with
//               their signs (bf16x2, exact) and write all six slices of the
//               chunk into a ring slot of shared memory in the canonical
//               no-swizzle K-major image; then fence.proxy.async and one
//               mbarrier arrive per warp.
// No D image goes through HBM: per determinant the kernel reads psi's digit
// words (from L2, the tile order keeps them resident) and writes G.
// The MMA loop runs K chunk outer, D slice, V slice inner; a ring slot holds
// one K chunk of a tile pair with its six slices (24 KB) and is released
// when its MMAs complete.
// Register cap: the 17 warps are spread over the four SM sub-partitions (16K
// registers each), five on one of them, so a thread may hold at most 96
// registers; bounds of 20 warps make the compiler keep to that.
__global__ void __launch_bounds__(kRegWarps * 32, 1) k_oz_fused(OzArgs A) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int KP = A.KP, R = A.ring;
  const int NP = A.NP;
  const uint32_t v_elems = (uint32_t)NP * KP;
  const int nch = KP / kChunkK;  // K chunks per tile pair
  const int64_t npairs = (A.ntiles + 1) / 2;
  __nv_bfloat16* sV = reinterpret_cast<__nv_bfloat16*>(smem);
  unsigned char* sD = reinterpret_cast<unsigned char*>(sV + kSlices * v_elems);
  uint64_t* full = reinterpret_cast<uint64_t*>(sD + (size_t)R * kSlotBytes);
  uint64_t* empty = full + kMaxRing;
  uint64_t* accfull = empty + kMaxRing;
  uint64_t* accempty = accfull + 1;
  uint64_t* done = accempty + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
  int* sVexp = reinterpret_cast<int*>(tslot + 2);  // [kM] row exponents of V
  // [kM] 2^(eV(p) + g0 + 1) per output pair, 0 where outside FP32's range
  float* sScale = reinterpret_cast<float*>(sVexp + kM);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  {
    const int4* src = reinterpret_cast<const int4*>(A.vslices);
    int4* dst = reinterpret_cast<int4*>(sV);
    const int n16 = (int)(kSlices * v_elems * 2 / 16);
    for (int i = tid; i < n16; i += blockDim.x) dst[i] = src[i];
    const int g1 = A.misc[0] + 1;
    for (int i = tid; i < NP; i += blockDim.x) {
      const int e = A.vexp[i];
      sVexp[i] = e;
      const int sc = e + g1;
      sScale[i] = (sc >= -126 && sc <= 127) ? pow2f(sc) : 0.0f;
    }
  }
  if (tid == 0) {
    for (int i = 0; i < R; ++i) {
      tc::mbar_init(&full[i], kProdWarps);
      tc::mbar_init(&empty[i], 1);
    }
    tc::mbar_init(accfull, 1);
    tc::mbar_init(accempty, kEpiWarps);
    tc::mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_proxy_async_smem();
  __syncthreads();
  if (warp == kMmaWarp) tc::tmem_alloc(tslot, kTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  // each CTA owns a contiguous run of tile pairs (in the super-block order of
  // tile_coords)
  const int64_t t_begin = npairs * blockIdx.x / gridDim.x;
  const int64_t t_end = npairs * (blockIdx.x + 1) / gridDim.x;

  if (warp >= kProdWarp0) {
    // producer thread: quarter qq (pairs 4 qq .. 4 qq + 3 of every K chunk)
    // of determinant d; a warp takes 8 consecutive beta columns.  The two
    // lanes of a quarter pair (qq, qq ^ 1; adjacent lanes) swap halves so
    // that each stores one whole 16-byte core-matrix row per slice: the even
    // lane the real row 2 dl, the odd lane the imaginary row 2 dl + 1, k =
    // 8 (qq >> 1) .. + 7.  Lane bits (qq & 1, d & 3, qq >> 1, d >> 2 of the
    // warp's 8) put rows 0..7 of one K core in every 8-lane phase of a
    // 16-byte store: 128 contiguous bytes, no bank conflicts.
    const int pt = tid - kProdWarp0 * 32;
    const int qq = ((lane >> 3) & 1) * 2 + (lane & 1);
    const int d = (pt >> 5) * 8 + (lane >> 4) * 4 + ((lane >> 1) & 3);
    const int tile = d >> 5, dl = d & 31;
    const bool odd = (qq & 1) != 0;
    const uint32_t lenb32 = (uint32_t)A.lenb;
    // byte offset of this thread's row in a slice region of a slot
    const uint32_t roff =
        (uint32_t)tile * (uint32_t)kChunkElems * 2u +
        tc::kmajor_offset(2 * dl + (odd ? 1 : 0), 8 * (qq >> 1), kChunkK) * 2u;
    const uint32_t sD0 = tc::smem_u32(sD);
    int slot = 0;
    uint32_t ph = 0;
    bool ok = true;
    for (int64_t t = t_begin; t < t_end && ok; ++t) {
      const int64_t ts = 2 * t + tile;
      int64_t ia64 = 0, ib064 = 0;
      const bool live_tile = ts < A.ntiles;
      if (live_tile) tile_coords(A, ts, ia64, ib064);
      const uint32_t ia = (uint32_t)ia64;
      const uint32_t ib = (uint32_t)ib064 + dl;
      const bool valid = live_tile && ib < lenb32;
      const int4* pa = reinterpret_cast<const int4*>(A.tabTA + (size_t)ia * KP + 4 * qq);
      const int4* pb = reinterpret_cast<const int4*>(A.tabTB + (size_t)ib * KP + 4 * qq);
      // this quarter's four table entries per spin (one 16-byte load each),
      // loaded one K chunk ahead so that a chunk's gathers wait for one
      // global round trip, not two
      int4 tan = make_int4(0, 0, 0, 0), tbn = tan;
      if (valid) {
        tan = __ldg(pa);
        tbn = __ldg(pb);
      }
      for (int c = 0; c < nch; ++c) {
        const int4 ta = tan, tb = tbn;
        if (valid && c + 1 < nch) {
          tan = __ldg(pa + 4 * (c + 1));
          tbn = __ldg(pb + 4 * (c + 1));
        }
        const int32_t cas[4] = {ta.x, ta.y, ta.z, ta.w};
        const int32_t cbs[4] = {tb.x, tb.y, tb.z, tb.w};
        uint32_t re[kDSlices][2], im[kDSlices][2];
#pragma unroll
        for (int jp = 0; jp < 2; ++jp) {
          uint32_t sum[2][kDSlices];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int32_t ca = cas[2 * jp + u], cb = cbs[2 * jp + u];
            uint4 a4 = make_uint4(0u, 0u, 0u, 0u), b4 = a4;
            uint2 a2 = make_uint2(0u, 0u), b2 = a2;
            if (ca) {
              const uint32_t idx = (uint32_t)(abs(ca) - 1) * lenb32 + ib;
              a4 = __ldg(A.pdA + idx);
              a2 = __ldg(A.pdB + idx);
            }
            if (cb) {
              const uint32_t idx = ia * lenb32 + (uint32_t)(abs(cb) - 1);
              b4 = __ldg(A.pdA + idx);
              b2 = __ldg(A.pdB + idx);
            }
            const uint32_t ma = ca < 0 ? 0x80008000u : 0u, mb = cb < 0 ? 0x80008000u : 0u;
#pragma unroll
            for (int k = 0; k < kDSlices; ++k) {
              const uint32_t x = digit_word(a4, a2, k) ^ ma, y = digit_word(b4, b2, k) ^ mb;
              const __nv_bfloat162 z = __hadd2(*reinterpret_cast<const __nv_bfloat162*>(&x),
                                               *reinterpret_cast<const __nv_bfloat162*>(&y));
              sum[u][k] = *reinterpret_cast<const uint32_t*>(&z);
            }
          }
#pragma unroll
          for (int k = 0; k < kDSlices; ++k) {
            re[k][jp] = __byte_perm(sum[0][k], sum[1][k], 0x5410u);
            im[k][jp] = __byte_perm(sum[0][k], sum[1][k], 0x7632u);
          }
        }
        // the slot must have been released by the MMAs of its last use
        if (!__all_sync(0xffffffffu, oz_wait(&empty[slot], ph ^ 1u, abort_flag, A.wait_cycles))) {
          if (lane == 0) oz_abort(abort_flag, A.err, 5);
          ok = false;
          break;
        }
        const uint32_t base = sD0 + (uint32_t)slot * (uint32_t)kSlotBytes + roff;
#pragma unroll
        for (int k = 0; k < kDSlices; ++k) {
          // the even lane keeps its real half and takes its partner's; the odd
          // lane keeps its imaginary half, which comes second in the row
          const uint32_t s0 = odd ? re[k][0] : im[k][0], s1 = odd ? re[k][1] : im[k][1];
          const uint32_t r0 = __shfl_xor_sync(0xffffffffu, s0, 1);
          const uint32_t r1 = __shfl_xor_sync(0xffffffffu, s1, 1);
          const uint32_t w0 = odd ? r0 : re[k][0], w1 = odd ? r1 : re[k][1];
          const uint32_t w2 = odd ? im[k][0] : r0, w3 = odd ? im[k][1] : r1;
          const uint32_t q = base + (uint32_t)k * (uint32_t)kPairChunkElems * 2u;
          asm volatile("st.shared.v4.b32 [%0], {%1,%2,%3,%4};" ::"r"(q), "r"(w0), "r"(w1),
                       "r"(w2), "r"(w3)
                       : "memory");
        }
        // generic-proxy writes -> visible to the tensor core (async proxy)
        tc::fence_proxy_async_smem();
        __syncwarp();
        const bool skip = A.skip_slot >= 0 && blockIdx.x == 0 && t == t_begin &&
                          c == A.skip_slot;  // test injection: this chunk never arrives
        if (lane == 0 && !skip) tc::mbar_arrive(&full[slot]);
        if (++slot == R) {
          slot = 0;
          ph ^= 1u;
        }
      }
    }
  } else if (warp == kMmaWarp) {
    // The whole warp runs the issue loop, so descriptors and counters stay
    // warp-uniform; lane 0 alone issues the MMAs and commits.  Levels,
    // accumulators and accumulate flags are compile-time after unrolling b
    // and a.
    const uint32_t elect = lane == 0 ? 1u : 0u;
    const uint32_t idesc = tc::make_idesc_bf16(kM, (uint32_t)NP);
    const uint32_t sbo = (uint32_t)KP * 16u;          // V: full-K rows
    const uint32_t sbo_c = (uint32_t)kChunkK * 16u;   // D chunk: 16-column rows
    // B = V slice descriptors of k-step 0; k-step c adds 256 bytes = 16 units
    uint64_t vdesc0[kSlices];
#pragma unroll
    for (int a = 0; a < kSlices; ++a)
      vdesc0[a] = tc::make_sdesc(tc::smem_u32(sV + (size_t)a * v_elems), 128, sbo);
    uint32_t accs[kAccs];
#pragma unroll
    for (int i = 0; i < kAccs; ++i) accs[i] = tmem + (uint32_t)(i * NP);
    const uint32_t sD0 = tc::smem_u32(sD);
    int64_t it = 0;
    int slot = 0;
    uint32_t ph = 0;
    bool ok = true;
    for (int64_t t = t_begin; t < t_end && ok; ++t, ++it) {
      // warp-uniform outcome of every wait
      if (!__all_sync(0xffffffffu,
                      oz_wait(accempty, (uint32_t)((it & 1) ^ 1), abort_flag, A.wait_cycles))) {
        if (elect) oz_abort(abort_flag, A.err, 2);
        ok = false;
        break;
      }
      tc::fence_after_sync();
      for (int c = 0; c < nch; ++c) {
        if (!__all_sync(0xffffffffu, oz_wait(&full[slot], ph, abort_flag, A.wait_cycles))) {
          if (elect) oz_abort(abort_flag, A.err, 3);
          ok = false;
          break;
        }
        tc::fence_after_sync();
        // slice b of the chunk: a 4 KB region of the slot (256 units)
        const uint64_t dd = tc::make_sdesc(sD0 + (uint32_t)slot * (uint32_t)kSlotBytes, 128,
                                           sbo_c);
        const uint64_t kb = (uint64_t)(16 * c);
        // the first MMA into each accumulator of the tile pair (first chunk,
        // b = 1, a <= 4) overwrites it
        const uint32_t first = c == 0 ? 1u : 0u;
#pragma unroll
        for (int b = 1; b <= kDSlices; ++b) {
          const uint64_t da = dd + (uint64_t)(256 * (b - 1));
#pragma unroll
          for (int a = 1; a <= kSlices; ++a) {
            if (a + b <= kMaxLevel) {
              const int ai = acc_of(a, b);
              const uint32_t accum = (b == 1 && a <= 4) ? (first ^ 1u) : 1u;
              tc::mma_bf16_if(accs[ai], da, vdesc0[a - 1] + kb, idesc, accum, elect);
            }
          }
        }
        if (elect) tc::mma_commit(&empty[slot]);
        __syncwarp();
        if (++slot == R) {
          slot = 0;
          ph ^= 1u;
        }
      }
      if (!ok) break;
      if (elect) tc::mma_commit(accfull);
      __syncwarp();
    }
    // every MMA issued above has completed before TMEM is released
    if (elect) {
      tc::mma_commit(done);
      // MMAs always complete: this wait ignores the abort flag
      if (!oz_wait_drain(done, 0, A.wait_cycles + kWaitCycles)) oz_abort(abort_flag, A.err, 6);
    }
    __syncwarp();
  } else if (warp < kEpiWarps) {
    const int quarter = warp & 3, cg = warp >> 2;
    const int row = 32 * quarter + lane;      // TMEM lane = MMA row
    const int half = row >> 6;                // slice tile of the pair
    const int det = (row & 63) >> 1;          // determinant in that tile
    const int part = row & 1;                 // 0 real, 1 imaginary
    const int cw = NP / 2;                    // pairs per column half (NP / 16 * 8)
    const int pbeg = cg * cw;
    const int nst = min(cw, A.P - A.p0 - pbeg);  // columns holding real pairs
    // D = 2^(g0 + 1) sum_b slice_b for every determinant (one global scale)
    const int colexp = A.misc[0] + 1;
    const int64_t pstride = A.lena * A.gld * 2;  // float2 elements per pair row
    int64_t it = 0;
    for (int64_t t = t_begin; t < t_end; ++t, ++it) {
      const int64_t ts = 2 * t + half;
      const bool live_tile = ts < A.ntiles;
      int64_t ia = 0, ib0 = 0;
      if (live_tile) tile_coords(A, ts, ia, ib0);
      const int64_t ib = ib0 + det;
      const bool live = live_tile && ib < A.lenb;
      const bool got = __all_sync(0xffffffffu,
                                  oz_wait(accfull, (uint32_t)(it & 1), abort_flag, A.wait_cycles));
      if (!got) {
        if (lane == 0) oz_abort(abort_flag, A.err, 4);
        break;
      }
      tc::fence_after_sync();
      const uint32_t base = tmem + ((uint32_t)(32 * quarter) << 16);
      // this lane's half of G[p][det]: (hi, lo) of the real or imaginary part
      float2* gp = reinterpret_cast<float2*>(A.G + ia * A.gld + (ib - A.c0)) + part +
                   (int64_t)(A.p0 + pbeg) * pstride;
      // Four columns at a time, software-pipelined: the TMEM loads of the
      // next four columns are in flight while these are combined and stored.
      // Per column the four level sums become an FP32 pair (h, l) by a chain
      // of exact two-sums (with one global scale a column's leading bits may
      // sit in level 4 or later, so no level is assumed to dominate; the
      // rounding errors are summed in l).  The pair is left unnormalised: the
      // scatter adds it in FP32-pair arithmetic, which absorbs l.
      uint32_t xa[16], xb[16];  // [level * 4 + column]
      auto load4 = [&](uint32_t (&x)[16], int pc) {
        uint32_t (&x0)[4] = *reinterpret_cast<uint32_t (*)[4]>(&x[0]);
        uint32_t (&x1)[4] = *reinterpret_cast<uint32_t (*)[4]>(&x[4]);
        uint32_t (&x2)[4] = *reinterpret_cast<uint32_t (*)[4]>(&x[8]);
        uint32_t (&x3)[4] = *reinterpret_cast<uint32_t (*)[4]>(&x[12]);
        tc::tmem_ld4_nowait(base + (uint32_t)pc, x0);
        tc::tmem_ld4_nowait(base + (uint32_t)(NP + pc), x1);
        tc::tmem_ld4_nowait(base + (uint32_t)(2 * NP + pc), x2);
        tc::tmem_ld4_nowait(base + (uint32_t)(3 * NP + pc), x3);
      };
      auto emit4 = [&](const uint32_t (&x)[16], int c0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float h, l, e2;
          two_sum(__uint_as_float(x[k]), __uint_as_float(x[4 + k]), h, l);
          two_sum(h, __uint_as_float(x[8 + k]), h, e2);
          l += e2;
          two_sum(h, __uint_as_float(x[12 + k]), h, e2);
          l += e2;
          const int pc = pbeg + c0 + k;
          // with the row exponent of V: 2^(eV(p) + g0 + 1), precomputed
          const float f = sScale[pc];
          float hs, ls;
          if (f != 0.0f) {
            hs = h * f;
            ls = l * f;
          } else {  // outside FP32's normal exponent range: two steps
            const int sc = sVexp[pc] + colexp;
            hs = scale2(h, sc);
            ls = scale2(l, sc);
          }
          if (live && c0 + k < nst) gp[(int64_t)(c0 + k) * pstride] = make_float2(hs, ls);
        }
      };
      // cw is a multiple of 8: the batches come in pairs
      load4(xa, pbeg);
      for (int c0 = 0; c0 < cw; c0 += 8) {
        tc::tmem_wait_ld_tied(xa);
        load4(xb, pbeg + c0 + 4);
        emit4(xa, c0);
        tc::tmem_wait_ld_tied(xb);
        if (c0 + 8 < cw) {
          load4(xa, pbeg + c0 + 8);
        } else {
          // every TMEM load of this warp has completed: release the
          // accumulators before the last four columns are stored
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(accempty);
        }
        emit4(xb, c0 + 4);
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, kTmemCols);
}


// ---- pre-pass: global exponent and the fixed-point copy of psi ------------
__device__ __forceinline__ int exp_of(double x) {
  // e with |x| < 2^e (frexp convention); kExpZero for 0, kExpNonFinite for
  // Inf and NaN
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7FF);
  if (be == 0x7FF) return kExpNonFinite;
  if (be == 0) return (b << 1) == 0 ? kExpZero : -1022;  // subnormals: bound
  return be - 1022;
}

__global__ void k_oz_rowexp(int64_t lenb, const double2* __restrict__ psi,
                            int32_t* __restrict__ rowexp) {
  __shared__ int red[256];
  const int64_t a = blockIdx.x;
  int e = kExpZero;
  for (int64_t b = threadIdx.x; b < lenb; b += blockDim.x) {
    const double2 v = psi[a * lenb + b];
    e = max(e, max(exp_of(v.x), exp_of(v.y)));
  }
  red[threadIdx.x] = e;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = max(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) rowexp[a] = red[0];
}

__global__ void k_oz_globalexp(int64_t lena, const int32_t* __restrict__ rowexp,
                               int32_t* __restrict__ misc) {
  __shared__ int red[256];
  int e = kExpZero;
  for (int64_t a = threadIdx.x; a < lena; a += blockDim.x) e = max(e, rowexp[a]);
  red[threadIdx.x] = e;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = max(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    // misc[1], the sticky error word, is left alone; misc[2] flags an input
    // holding Inf or NaN (the scatter then writes NaN, as FP64 would)
    const int nonfinite = red[0] >= kExpNonFinite ? 1 : 0;
    misc[0] = nonfinite ? 0 : red[0];
    misc[2] = nonfinite;
  }
}

// The six balanced base-256 digits of x = round(v 2^(47 - g0)), |x| <= 2^47:
// digit b (b = 1..5) = floor(r / 2^k + 1/2) with k = 8 (6 - b) and r the
// remainder so far (|r| <= 128 2^k, so the digit lies in [-128, 128]); the
// last digit is the final remainder.  Returned as floats digit * 2^-8b.
// A small integer (|d| < 2^22) as a float, exactly, without a conversion
// instruction: the bits of 1.5 * 2^23 + d, minus 1.5 * 2^23.
__device__ __forceinline__ float small_int_float(int d) {
  return __int_as_float(0x4B400000 + d) - 12582912.0f;
}

__device__ __forceinline__ void psi_digits(long long x, float (&f)[kDSlices]) {
#pragma unroll
  for (int b = 1; b < kDSlices; ++b) {
    const int k = 8 * (kDSlices - b);
    const long long dgt = (x + (1ll << (k - 1))) >> k;  // in [-128, 128]
    x -= dgt << k;
    f[b - 1] = small_int_float((int)dgt) * __int_as_float((127 - 8 * b) << 23);
  }
  f[kDSlices - 1] = small_int_float((int)x) * __int_as_float((127 - 8 * kDSlices) << 23);
}

// v * 2^e rounded to the nearest integer, ties to even, built from the bits
// of v with integer operations only (GB300 runs FP64 multiplies and double
// conversions at a small fraction of its integer rate).  The caller keeps
// |v| < 2^(47 - e), so the result is below 2^47; v is finite.
__device__ __forceinline__ long long fixed_rn(double v, int e) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int be = (int)((bits >> 52) & 0x7FF);
  unsigned long long m = bits & 0xFFFFFFFFFFFFFull;
  int s = e - 1074;  // subnormal: m * 2^-1074
  if (be) {
    m |= 1ull << 52;
    s = e + be - 1075;
  }
  unsigned long long q;
  if (s >= 0) {
    q = m << s;
  } else if (s <= -64) {
    q = 0;
  } else {
    const int r = -s;
    q = m >> r;
    const unsigned long long rem = m & ((1ull << r) - 1ull), half = 1ull << (r - 1);
    if (rem > half || (rem == half && (q & 1ull))) ++q;
  }
  return (bits >> 63) ? -(long long)q : (long long)q;
}

// The digit planes of psi at the global exponent g0: pdA[i] = digits 1-4,
// pdB[i] = digits 5-6, each digit a bf16x2 (real, imaginary); exact.
__global__ void k_oz_digits(int64_t n, const double2* __restrict__ psi,
                            const int32_t* __restrict__ misc, uint4* __restrict__ pdA,
                            uint2* __restrict__ pdB) {
  const int g0 = misc[0];
  const bool skip = misc[2] != 0;  // non-finite input: the output is NaN anyway
  // psi * 2^(47 - g0), |psi| < 2^g0, as 47-bit fixed point
  const int e = 47 - g0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float fr[kDSlices] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, fi[kDSlices] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (!skip) {
      const double2 v = psi[i];
      psi_digits(fixed_rn(v.x, e), fr);
      psi_digits(fixed_rn(v.y, e), fi);
    }
    uint32_t wd[kDSlices];
#pragma unroll
    for (int k = 0; k < kDSlices; ++k) {
      const __nv_bfloat162 h = __floats2bfloat162_rn(fr[k], fi[k]);  // exact
      wd[k] = *reinterpret_cast<const uint32_t*>(&h);
    }
    pdA[i] = make_uint4(wd[0], wd[1], wd[2], wd[3]);
    pdB[i] = make_uint2(wd[4], wd[5]);
  }
}

// ---- scatter in FP32-pair arithmetic ----------------------------------------
__device__ __forceinline__ void df_add(float& h, float& l, float bh, float bl) {
  const float s = h + bh;
  const float v = s - h;
  float e = (h - (s - v)) + (bh - v);
  e += l + bl;
  h = s + e;
  l = e - (h - s);
}

__device__ __forceinline__ double2 zmul2(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Column-block scatter with the beta part read from the block's CSR list:
// the alpha part only for targets inside the block (all pairs), the beta part
// only for the (pair, source) entries whose source lies in the block.  Same
// sums as k_oz_scatter over the same block, without scanning every pair of
// every target once per block.
__global__ void __launch_bounds__(256) k_oz_scatter_csr(
    int P, int64_t lena, int64_t lenb, int64_t c0, int64_t w, int64_t gld,
    const int32_t* __restrict__ tabA, const int32_t* __restrict__ boff,
    const int2* __restrict__ bent, const float4* __restrict__ G,
    const double2* __restrict__ psi, double2 alpha, double2 beta, int init,
    const int32_t* __restrict__ misc, double2* __restrict__ sigma, int64_t a0) {
  const int64_t a = a0 + blockIdx.y;
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= lenb) return;
  if (misc[2]) {  // psi holds Inf or NaN
    sigma[a * lenb + b] = make_double2(CUDART_NAN, CUDART_NAN);
    return;
  }
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  if (b >= c0 && b < c0 + w) {
    for (int p = 0; p < P; ++p) {
      const int32_t ca = tabA[(int64_t)p * lena + a];
      if (ca) {
        float4 g = G[((int64_t)p * lena + (abs(ca) - 1)) * gld + (b - c0)];
        if (ca < 0) g = make_float4(-g.x, -g.y, -g.z, -g.w);
        df_add(rh, rl, g.x, g.y);
        df_add(ih, il, g.z, g.w);
      }
    }
  }
  const int32_t e1 = boff[b + 1];
  for (int32_t e = boff[b]; e < e1; ++e) {
    const int2 en = bent[e];
    float4 g = G[((int64_t)en.x * lena + a) * gld + (abs(en.y) - 1)];
    if (en.y < 0) g = make_float4(-g.x, -g.y, -g.z, -g.w);
    df_add(rh, rl, g.x, g.y);
    df_add(ih, il, g.z, g.w);
  }
  const int64_t I = a * lenb + b;
  const double2 acc = make_double2((double)rh + (double)rl, (double)ih + (double)il);
  double2 out = zmul2(alpha, acc);
  if (init) {
    if (beta.x != 0.0 || beta.y != 0.0) {
      const double2 t = zmul2(beta, psi[I]);
      out.x += t.x;
      out.y += t.y;
    }
  } else {
    const double2 s0 = sigma[I];
    out.x += s0.x;
    out.y += s0.y;
  }
  sigma[I] = out;
}

// sigma[I] (init: beta psi[I] +, else sigma[I] +) alpha * the contributions of
// the beta-column block [c0, c0 + w) held in G ([P][lena][w]): the alpha part
// of targets in the block, the beta part of every target whose source column
// lies in the block (G rows have gld entries).  One block covering all
// columns is the whole apply.
__global__ void __launch_bounds__(256) k_oz_scatter(
    int P, int64_t lena, int64_t lenb, int64_t c0, int64_t w, int64_t gld,
    const int32_t* __restrict__ tabA,
    const int32_t* __restrict__ tabB, const float4* __restrict__ G,
    const double2* __restrict__ psi, double2 alpha, double2 beta, int init,
    const int32_t* __restrict__ misc, double2* __restrict__ sigma, int64_t a0) {
  const int64_t a = a0 + blockIdx.y;
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= lenb) return;
  if (misc[2]) {  // psi holds Inf or NaN
    sigma[a * lenb + b] = make_double2(CUDART_NAN, CUDART_NAN);
    return;
  }
  const bool inblk = b >= c0 && b < c0 + w;
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  for (int p = 0; p < P; ++p) {
    const int32_t ca = tabA[(int64_t)p * lena + a];
    if (ca && inblk) {
      float4 g = G[((int64_t)p * lena + (abs(ca) - 1)) * gld + (b - c0)];
      if (ca < 0) g = make_float4(-g.x, -g.y, -g.z, -g.w);
      df_add(rh, rl, g.x, g.y);
      df_add(ih, il, g.z, g.w);
    }
    const int32_t cb = tabB[(int64_t)p * lenb + b];
    if (cb) {
      const int64_t J = abs(cb) - 1;
      if (J >= c0 && J < c0 + w) {
        float4 g = G[((int64_t)p * lena + a) * gld + (J - c0)];
        if (cb < 0) g = make_float4(-g.x, -g.y, -g.z, -g.w);
        df_add(rh, rl, g.x, g.y);
        df_add(ih, il, g.z, g.w);
      }
    }
  }
  const int64_t I = a * lenb + b;
  const double2 acc = make_double2((double)rh + (double)rl, (double)ih + (double)il);
  double2 out = zmul2(alpha, acc);
  if (init) {
    if (beta.x != 0.0 || beta.y != 0.0) {
      const double2 t = zmul2(beta, psi[I]);
      out.x += t.x;
      out.y += t.y;
    }
  } else {
    const double2 s0 = sigma[I];
    out.x += s0.x;
    out.y += s0.y;
  }
  sigma[I] = out;
}

// tabT[s][q] = tab[q][s] for q < P, 0 for P <= q < KP.
__global__ void k_oz_transpose_tab(int P, int KP, int64_t len, const int32_t* __restrict__ tab,
                                   int32_t* __restrict__ tabT) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= len * KP) return;
  const int64_t s = i / KP;
  const int q = (int)(i - s * KP);
  tabT[i] = q < P ? tab[(int64_t)q * len + s] : 0;
}

// ---- host ---------------------------------------------------------------------
// Shape of the tensor-core form for P pairs: K = KP (pairs rounded up to 16),
// output pairs in npass passes of NP rows (four level accumulators of NP TMEM
// columns, NP <= 128; five NP x KP V slices in shared memory beside a ring of
// at least two 24 KB ring slots).  False when the sector does not fit (FP64
// kernels).
static bool oz_shape(int P, int smax, int& KP, int& npass, int& NP, size_t& fixed) {
  KP = (P + 15) / 16 * 16;
  if (KP > 192) return false;  // five NP x KP V slices beside two slots
  npass = KP <= kM ? 1 : 2;
  NP = ((P + npass - 1) / npass + 15) / 16 * 16;
  if (NP > kM) return false;
  fixed = sizeof(__nv_bfloat16) * (size_t)kSlices * NP * KP +
          sizeof(uint64_t) * (2 * kMaxRing + 3) + 16 + sizeof(int) * kM + sizeof(float) * kM;
  return fixed + 2 * (size_t)kSlotBytes <= (size_t)smax;
}

static int plan_create(fqegpu_ham h) {
  int dev = 0, smax = 0;
  FQE_CUDA(cudaGetDevice(&dev));
  FQE_CUDA(cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const int P = h->P;
  int KP = 0, npass = 0, NP = 0;
  size_t fixed = 0;
  if (!oz_shape(P, smax, KP, npass, NP, fixed)) {
    set_error("pair count %d does not fit the tensor-core contraction", P);
    return FQEGPU_ERR_UNSUPPORTED;
  }
  auto* pl = new (std::nothrow) OzakiPlan();
  if (!pl) {
    set_error("host allocation failed");
    return FQEGPU_ERR_NOMEM;
  }
  h->oz = pl;
  pl->P = P;
  pl->KP = KP;
  pl->npass = npass;
  pl->NP = NP;
  const size_t vel = (size_t)NP * KP;  // V slice of one pass: NP rows (pairs) x KP
  std::vector<__nv_bfloat16> sl((size_t)npass * kSlices * vel, __float2bfloat16(0.0f));
  std::vector<int32_t> vexp((size_t)npass * NP, 0);
  for (int p = 0; p < P; ++p) {
    const int pass = p / NP, r = p - pass * NP;
    double mx = 0.0;
    for (int q = 0; q < P; ++q) mx = std::max(mx, std::fabs(h->vpair[(size_t)p * P + q]));
    if (mx == 0.0) continue;
    int e;
    std::frexp(mx, &e);  // mx < 2^e
    vexp[(size_t)pass * NP + r] = e;
    for (int q = 0; q < P; ++q) {
      const double v = h->vpair[(size_t)p * P + q];
      const double y = std::floor(std::ldexp(std::fabs(v), 40 - e) + 0.5);
      const uint64_t m = std::min<uint64_t>((uint64_t)y, (1ull << 40) - 1ull);
      for (int k = 1; k <= kSlices; ++k) {
        const uint32_t byte = (uint32_t)((m >> (40 - 8 * k)) & 0xFFu);
        const float f = std::ldexp((float)byte, -8 * k) * (v < 0 ? -1.0f : 1.0f);
        sl[((size_t)pass * kSlices + (k - 1)) * vel + tc::kmajor_offset(r, q, KP)] =
            __float2bfloat16(f);
      }
    }
  }
  FQE_CUDA(dev_alloc(&pl->d_vslices, sizeof(__nv_bfloat16) * sl.size()));
  FQE_CUDA(cudaMemcpy(pl->d_vslices, sl.data(), sizeof(__nv_bfloat16) * sl.size(),
                      cudaMemcpyHostToDevice));
  FQE_CUDA(dev_alloc(&pl->d_vexp, sizeof(int32_t) * vexp.size()));
  FQE_CUDA(cudaMemcpy(pl->d_vexp, vexp.data(), sizeof(int32_t) * vexp.size(),
                      cudaMemcpyHostToDevice));
  const int64_t lena = h->g->a.len, lenb = h->g->b.len, N = lena * lenb;
  // beta-column blocks: G (16 P bytes per determinant) of a block within the
  // handle's scratch limit
  const int64_t per_col = (int64_t)(16 * P) * lena;
  int64_t wb = h->scratch_limit / std::max<int64_t>(per_col, 1);
  if (wb >= lenb) {
    wb = lenb;  // one block: G is [P][lena][lenb]
  } else {
    wb = std::max<int64_t>(kDets, wb / kDets * kDets);
  }
  pl->wb = wb;
  FQE_CUDA(dev_alloc(&pl->d_pdA, sizeof(uint4) * N));
  FQE_CUDA(dev_alloc(&pl->d_pdB, sizeof(uint2) * N));
  FQE_CUDA(dev_alloc(&pl->d_rowexp, sizeof(int32_t) * lena));
  FQE_CUDA(dev_alloc(&pl->d_misc, sizeof(int32_t) * 4));
  FQE_CUDA(cudaMemset(pl->d_misc, 0, sizeof(int32_t) * 4));
  FQE_CUDA(cudaHostAlloc(&pl->h_err, sizeof(int32_t), cudaHostAllocDefault));
  *pl->h_err = 0;
  FQE_CUDA(cudaEventCreateWithFlags(&pl->err_ev, cudaEventDisableTiming));
  FQE_CUDA(dev_alloc(&pl->d_G, sizeof(float4) * (size_t)P * lena * wb));
  {
    const int32_t* ta = ham_tabA(h);
    const int32_t* tb = ham_tabB(h);
    FQE_CUDA(dev_alloc(&pl->d_tabTA, sizeof(int32_t) * (size_t)lena * KP));
    FQE_CUDA(dev_alloc(&pl->d_tabTB, sizeof(int32_t) * (size_t)lenb * KP));
    k_oz_transpose_tab<<<(unsigned)((lena * KP + 255) / 256), 256>>>(P, KP, lena, ta,
                                                                     pl->d_tabTA);
    k_oz_transpose_tab<<<(unsigned)((lenb * KP + 255) / 256), 256>>>(P, KP, lenb, tb,
                                                                     pl->d_tabTB);
    FQE_CUDA(cudaGetLastError());
    FQE_CUDA(cudaDeviceSynchronize());
  }
  if (wb < lenb) {
    // per block, for every target column, the (pair, source) entries whose
    // beta source lies in the block, in pair order
    const int32_t* tb = ham_tabB(h);
    std::vector<int32_t> tab((size_t)P * lenb);
    FQE_CUDA(cudaMemcpy(tab.data(), tb, sizeof(int32_t) * tab.size(), cudaMemcpyDeviceToHost));
    const int64_t nblk = (lenb + wb - 1) / wb;
    const size_t row = (size_t)lenb + 1;
    std::vector<int32_t> off((size_t)nblk * row, 0);
    // counting sort by (block of the source, target column), pair order kept
    for (int64_t b = 0; b < lenb; ++b)
      for (int p = 0; p < P; ++p) {
        const int32_t cb = tab[(size_t)p * lenb + b];
        if (cb) ++off[(size_t)((std::abs(cb) - 1) / wb) * row + b + 1];
      }
    for (size_t i = 1; i < off.size(); ++i) off[i] += off[i - 1];  // [k][0] counts nothing
    std::vector<int2> ent((size_t)off.back());
    std::vector<int32_t> cur(off);
    for (int64_t b = 0; b < lenb; ++b)
      for (int p = 0; p < P; ++p) {
        const int32_t cb = tab[(size_t)p * lenb + b];
        if (!cb) continue;
        const int64_t src = std::abs(cb) - 1, k = src / wb;
        const int32_t v = (int32_t)(src - k * wb + 1);
        ent[(size_t)cur[(size_t)k * row + b]++] = make_int2(p, cb > 0 ? v : -v);
      }
    FQE_CUDA(dev_alloc(&pl->d_boff, sizeof(int32_t) * off.size()));
    FQE_CUDA(cudaMemcpy(pl->d_boff, off.data(), sizeof(int32_t) * off.size(),
                        cudaMemcpyHostToDevice));
    FQE_CUDA(dev_alloc(&pl->d_bent, sizeof(int2) * std::max<size_t>(ent.size(), 1)));
    if (!ent.empty())
      FQE_CUDA(cudaMemcpy(pl->d_bent, ent.data(), sizeof(int2) * ent.size(),
                          cudaMemcpyHostToDevice));
  }
  FQE_CUDA(cudaDeviceGetAttribute(&pl->nsm, cudaDevAttrMultiProcessorCount, dev));
  // as many ring slots as shared memory holds after the V slices
  pl->ring = (int)std::min<size_t>(kMaxRing, ((size_t)smax - fixed) / kSlotBytes);
  pl->smem = fixed + (size_t)pl->ring * kSlotBytes;
  // the attribute belongs to the kernel, not to this plan: set the device
  // maximum so plans of different sectors (different ring sizes) can coexist
  FQE_CUDA(cudaFuncSetAttribute(k_oz_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
  return FQEGPU_OK;
}

// Blocking check of the tensor-core path's sticky error word: waits for
// `st`, reads the word, clears it, and reports FQEGPU_ERR_TIMEOUT when a
// bounded wait of any apply since the last check gave up.
int ozaki_check(fqegpu_ham h, cudaStream_t st) {
  OzakiPlan* pl = h->oz;
  if (!pl) return FQEGPU_OK;
  FQE_CUDA(cudaStreamSynchronize(st));
  if (pl->err_pending) FQE_CUDA(cudaEventSynchronize(pl->err_ev));
  pl->err_pending = false;
  int32_t v = 0;
  FQE_CUDA(cudaMemcpy(&v, pl->d_misc + 1, sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (v != 0) {
    FQE_CUDA(cudaMemset(pl->d_misc + 1, 0, sizeof(int32_t)));
    *pl->h_err = 0;
    set_error("tensor-core contraction: a bounded wait gave up (role %d)", v);
    return FQEGPU_ERR_TIMEOUT;
  }
  return FQEGPU_OK;
}

// Non-blocking poll: if the last apply's error word has reached the host and
// is set, clear it and report the timeout now.
static int ozaki_poll(OzakiPlan* pl, cudaStream_t st) {
  if (!pl->err_pending) return FQEGPU_OK;
  const cudaError_t q = cudaEventQuery(pl->err_ev);
  if (q == cudaErrorNotReady) return FQEGPU_OK;
  FQE_CUDA(q);
  pl->err_pending = false;
  const int32_t v = *pl->h_err;
  if (v == 0) return FQEGPU_OK;
  *pl->h_err = 0;
  FQE_CUDA(cudaMemsetAsync(pl->d_misc + 1, 0, sizeof(int32_t), st));
  set_error("tensor-core contraction of an earlier apply: a bounded wait gave up (role %d)", v);
  return FQEGPU_ERR_TIMEOUT;
}

int ozaki_prepare(fqegpu_ham h) {
  if (h->zero || h->onebody || !h->real || h->P > 192) return FQEGPU_ERR_UNSUPPORTED;
  if (h->g->a.len > 65535) return FQEGPU_ERR_UNSUPPORTED;
  if (!h->oz) {
    const int s = plan_create(h);
    if (s == FQEGPU_ERR_UNSUPPORTED && !h->oz) return FQEGPU_ERR_UNSUPPORTED;
    FQE_TRY(s);
  }
  return FQEGPU_OK;
}

bool ozaki_runs_fp64(fqegpu_ham h) { return h->oz && h->oz->use_fp64; }

int ozaki_tuning_key(fqegpu_ham h) {
  return h->oz ? (h->oz->super << 1) | (h->oz->use_fp64 ? 1 : 0) : -1;
}

int ozaki_set_tuning(fqegpu_ham h, int super_tiles, int use_fp64) {
  FQE_TRY(ozaki_prepare(h));
  if (super_tiles > 0) h->oz->super = super_tiles;
  h->oz->use_fp64 = use_fp64 != 0;
  return FQEGPU_OK;
}

int ozaki_set_test_injection(fqegpu_ham h, long long wait_cycles, int skip_slot) {
  FQE_TRY(ozaki_prepare(h));
  h->oz->wait_cycles = wait_cycles > 0 ? wait_cycles : kWaitCycles;
  h->oz->skip_slot = skip_slot;
  return FQEGPU_OK;
}

void ozaki_destroy(fqegpu_ham h) {
  OzakiPlan* pl = h->oz;
  if (!pl) return;
  cudaFree(pl->d_vslices);
  cudaFree(pl->d_vexp);
  cudaFree(pl->d_pdA);
  cudaFree(pl->d_pdB);
  cudaFree(pl->d_rowexp);
  cudaFree(pl->d_misc);
  cudaFree(pl->d_G);
  cudaFree(pl->d_tabTA);
  cudaFree(pl->d_tabTB);
  cudaFree(pl->d_boff);
  cudaFree(pl->d_bent);
  if (pl->h_err) cudaFreeHost(pl->h_err);
  if (pl->err_ev) cudaEventDestroy(pl->err_ev);
  delete pl;
  h->oz = nullptr;
}

int apply_ozaki(fqegpu_ham h, const double2* psi, double2* sigma, double2 alpha,
                double2 beta, cudaStream_t st, HostOut* out) {
  // The split needs a real pair matrix whose shape fits the kernels (P <= 192,
  // shared memory); other operators run the FP64 kernels on the GPU.
  if (h->zero || h->onebody || !h->real || h->P > 192)
    return apply_fp64(h, psi, sigma, alpha, beta, st);
  const fqegpu_graph_s* g = h->g;
  const int64_t lena = g->a.len, lenb = g->b.len, N = lena * lenb;
  if (lena > 65535) {
    set_error("alpha string space of %lld exceeds the 65535 rows one launch covers",
              (long long)lena);
    return FQEGPU_ERR_UNSUPPORTED;
  }
  {
    const int s = ozaki_prepare(h);
    if (s == FQEGPU_ERR_UNSUPPORTED) return apply_fp64(h, psi, sigma, alpha, beta, st);
    FQE_TRY(s);
  }
  if (h->oz->use_fp64) return apply_fp64(h, psi, sigma, alpha, beta, st);
  OzakiPlan* pl = h->oz;
  if (!h->defer_check) FQE_TRY(ozaki_poll(pl, st));
  const int32_t* tabA = ham_tabA(h);
  const int32_t* tabB = ham_tabB(h);
  h->events_used = 0;
  FQE_TRY(stage_mark(h, 0, 0, st));
  k_oz_rowexp<<<(unsigned)lena, 256, 0, st>>>(lenb, psi, pl->d_rowexp);
  k_oz_globalexp<<<1, 256, 0, st>>>(lena, pl->d_rowexp, pl->d_misc);
  k_oz_digits<<<kNumSMs * 8, 256, 0, st>>>(N, psi, pl->d_misc, pl->d_pdA, pl->d_pdB);
  FQE_CUDA(cudaGetLastError());
  OzArgs A;
  A.P = pl->P;
  A.KP = pl->KP;
  A.ring = pl->ring;
  A.NP = pl->NP;
  A.lena = lena;
  A.lenb = lenb;
  A.gld = pl->wb;
  A.tabA = tabA;
  A.tabB = tabB;
  A.pdA = pl->d_pdA;
  A.pdB = pl->d_pdB;
  A.misc = pl->d_misc;
  A.G = pl->d_G;
  A.tabTA = pl->d_tabTA;
  A.tabTB = pl->d_tabTB;
  A.err = pl->d_misc + 1;
  A.wait_cycles = pl->wait_cycles;
  A.skip_slot = pl->skip_slot;
  A.super = pl->super;
  const size_t vel = (size_t)pl->NP * pl->KP;
  const double2 al = zmul_host(alpha, h->phase);
  int blk = 0;
  for (int64_t c0 = 0; c0 < lenb; c0 += pl->wb, ++blk) {
    const int64_t w = std::min<int64_t>(pl->wb, lenb - c0);
    A.c0 = c0;
    A.nb = (int)((w + kDets - 1) / kDets);
    A.ntiles = lena * (int64_t)A.nb;
    // stage 0 -> 1: the digit pre-pass (first block only)
    if (blk > 0) FQE_TRY(stage_mark(h, blk, 0, st));
    FQE_TRY(stage_mark(h, blk, 1, st));
    const int grid = (int)std::min<int64_t>(pl->nsm, (A.ntiles + 1) / 2);
    for (int pass = 0; pass < pl->npass; ++pass) {
      A.p0 = pass * pl->NP;
      A.vslices = pl->d_vslices + (size_t)pass * kSlices * vel;
      A.vexp = pl->d_vexp + (size_t)pass * pl->NP;
      k_oz_fused<<<grid, kThreads, pl->smem, st>>>(A);
      FQE_CUDA(cudaGetLastError());
    }
    FQE_TRY(stage_mark(h, blk, 2, st));
    // the last block's scatter leaves sigma final: with a host output it runs
    // in row chunks, each copied out as soon as it is written
    const bool last = c0 + pl->wb >= lenb;
    const int nchunk = (out && out->h_sigma && last) ? (int)std::min<int64_t>(kOutChunks, lena) : 1;
    for (int k = 0; k < nchunk; ++k) {
      const int64_t a0 = lena * k / nchunk, a1 = lena * (k + 1) / nchunk;
      dim3 sg((unsigned)((lenb + 255) / 256), (unsigned)(a1 - a0));
      if (pl->d_boff)
        k_oz_scatter_csr<<<sg, 256, 0, st>>>(pl->P, lena, lenb, c0, w, pl->wb, tabA,
                                             pl->d_boff + (size_t)blk * (lenb + 1), pl->d_bent,
                                             pl->d_G, psi, al, beta, blk == 0 ? 1 : 0,
                                             pl->d_misc, sigma, a0);
      else
        k_oz_scatter<<<sg, 256, 0, st>>>(pl->P, lena, lenb, c0, w, pl->wb, tabA, tabB,
                                         pl->d_G, psi, al, beta, blk == 0 ? 1 : 0, pl->d_misc,
                                         sigma, a0);
      FQE_CUDA(cudaGetLastError());
      if (nchunk > 1) {
        FQE_CUDA(cudaEventRecord(out->ev[k], st));
        FQE_CUDA(cudaStreamWaitEvent(out->copy, out->ev[k], 0));
        FQE_CUDA(cudaMemcpyAsync(out->h_sigma + a0 * lenb, sigma + a0 * lenb,
                                 sizeof(double2) * (size_t)((a1 - a0) * lenb),
                                 cudaMemcpyDeviceToHost, out->copy));
        out->issued = true;
      }
    }
    FQE_TRY(stage_mark(h, blk, 3, st));
  }
  if (h->defer_check) return FQEGPU_OK;  // recorded into a graph: checked by its owner
  // no host synchronisation: the sticky error word travels to pinned memory
  // behind the apply; the next apply polls it, fqegpu_ham_check waits for it
  FQE_CUDA(cudaMemcpyAsync(pl->h_err, pl->d_misc + 1, sizeof(int32_t), cudaMemcpyDeviceToHost,
                           st));
  FQE_CUDA(cudaEventRecord(pl->err_ev, st));
  pl->err_pending = true;
  return FQEGPU_OK;
}

}  // namespace fqegpu
