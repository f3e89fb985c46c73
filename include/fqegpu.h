/*
 * fqegpu — C ABI of the GB300 (sm_103a) implementation of the OpenFermion-FQE
 * restricted H·psi path.  Plain pointers and sizes only; no CUDA or PyTorch
 * types appear in a signature (streams are passed as `void*` holding a
 * cudaStream_t, NULL = the legacy default stream).
 *
 * Memory conventions
 *   - psi / sigma / dvec arrays are complex128, stored as interleaved
 *     (re, im) doubles, C-order, alpha-major: coeff[a * lenb + b], exactly the
 *     layout of FqeData.coeff (fqe_data.py:106).
 *   - "d_" arguments are device pointers owned by the caller; "h_" arguments
 *     are host pointers owned by the caller.  Integrals are always host arrays
 *     in the reference's own layout (they are tiny and are prepared on the
 *     host, as fqe_data.py:691-693 prepares them).
 *   - Handles (graph, hamiltonian, workspace) own their device memory and are
 *     released with the matching *_destroy call.
 *
 * Ordering: a Hamiltonian handle owns one apply's workspace (dvec blocks,
 * tensor-core plan, staging buffer), so calls on the same handle must be
 * ordered (one stream, or synchronised between streams); different handles
 * and graphs are independent and may run on different streams or threads.
 *
 * Errors: every entry point returns an fqegpu_status; nothing exits, traps or
 * prints.  The text of the last error of the calling thread is available from
 * fqegpu_last_error().  The reference instead exits from safe_malloc
 * (lib/macros.c:25-46) and returns void from its kernels.
 */
#ifndef FQEGPU_H
#define FQEGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  FQEGPU_OK = 0,
  FQEGPU_ERR_INVALID = 1,     /* bad shape / argument (reference: ValueError) */
  FQEGPU_ERR_NOMEM = 2,       /* device or host allocation failed            */
  FQEGPU_ERR_CUDA = 3,        /* CUDA runtime error (text in last_error)     */
  FQEGPU_ERR_UNSUPPORTED = 4, /* valid request this library does not handle  */
  FQEGPU_ERR_TIMEOUT = 5,     /* a bounded device wait gave up               */
  FQEGPU_ERR_NUMERIC = 6,     /* non-finite value or series did not converge */
} fqegpu_status;

/* Contraction arithmetic of fqegpu_apply / fqegpu_taylor. */
typedef enum {
  FQEGPU_PREC_FP64 = 0,   /* plain FP64: the drop-in, matches the reference  */
  FQEGPU_PREC_OZAKI = 1,  /* FP64 operands split into BF16 slices on the
                             tcgen05 tensor cores, FP32 accumulation,
                             compensated recombination (real integrals) */
} fqegpu_precision;

typedef struct fqegpu_graph_s *fqegpu_graph;
typedef struct fqegpu_ham_s *fqegpu_ham;

/* ---- library ------------------------------------------------------------ */
int fqegpu_version(void);
/* Copies the last error text of the calling thread (NUL terminated). */
int fqegpu_last_error(char *buf, int buflen);
/* Blocks until all work on `stream` is done; reports asynchronous errors. */
int fqegpu_sync(void *stream);

/* ---- K1: string graph ---------------------------------------------------
 * Replaces FciGraph.__init__ (fci_graph.py:108-154) and the natives it calls:
 * lexicographic_bitstring_generator (lib/bitstring.c:29-45),
 * calculate_Z_matrix (lib/fci_graph.c:27-54), calculate_string_address
 * (lib/fci_graph.c:136-147), build_mapping_strings (lib/fci_graph.c:76-121)
 * and map_deexc (lib/fci_graph.c:57-73).  All tables are built on the device.
 * norb <= 63, 0 <= nalpha, nbeta <= norb (fci_graph.py:124-137 checks). */
int fqegpu_graph_create(int norb, int nalpha, int nbeta, void *stream,
                        fqegpu_graph *out);
int fqegpu_graph_destroy(fqegpu_graph g);
/* lena, lenb, ndexca = nalpha*(norb-nalpha+1), ndexcb. */
int fqegpu_graph_dims(fqegpu_graph g, int64_t *lena, int64_t *lenb,
                      int *ndexca, int *ndexcb);
/* Copy-outs of the device tables in the reference's formats (spin 0 = alpha,
 * 1 = beta): strings uint64[len] (FciGraph._astr), Z int32[nele][norb]
 * (_get_Z_matrix), dexc int32[len][ndexc][3] (FciGraph._dexca),
 * map lengths int32[norb][norb] and maps int32[sum lengths][3], the
 * concatenation in (i, j) i-major order of FciGraph._alpha_map[(i, j)]. */
int fqegpu_graph_strings(fqegpu_graph g, int spin, uint64_t *h_out);
int fqegpu_graph_zmatrix(fqegpu_graph g, int spin, int32_t *h_out);
int fqegpu_graph_dexc(fqegpu_graph g, int spin, int32_t *h_out);
int fqegpu_graph_map_lengths(fqegpu_graph g, int spin, int32_t *h_out);
int fqegpu_graph_maps(fqegpu_graph g, int spin, int32_t *h_out);

/* ---- restricted Hamiltonian ----------------------------------------------
 * Prepares (h1, h2) of a RestrictedHamiltonian (restricted_hamiltonian.py)
 * for one sector: h1' = h1 - sum_k h2'[i,k,k,j], h2'[i,k,j,l] = -h2[i,j,k,l]
 * (fqe_data.py:691-693), with the one-body part folded into the pair matrix as
 * h1'[ij] delta_kl / N_e.  h_h1: complex128 [norb][norb] (may be NULL),
 * h_h2: complex128 [norb]^4 (may be NULL: one-body operator, the
 * _apply_array_spatial1 case, fqe_data.py:477-531).  The pair space is
 * compressed to norb(norb+1)/2 when the tensors have the real-orbital pair
 * symmetries, as fqe_data.py:658-681 does for real integrals. */
int fqegpu_ham_create(fqegpu_graph g, const double *h_h1, const double *h_h2,
                      void *stream, fqegpu_ham *out);
/* Spin-orbital (generalised) one- and two-body operator of the sector:
 * h_h1 complex128 [2 norb][2 norb] (may be NULL), h_h2 complex128 [2 norb]^4
 * (may be NULL: one-body), alpha spin orbitals first, in the reference's
 * layouts.  Replaces FqeData._apply_array_spin12_lm (fqe_data.py:743-773:
 * lm_apply_array12_same_spin_opt with the alpha-alpha and the beta-beta
 * blocks, lm_apply_array12_diff_spin_opt with h2'[a,a,b,b] + h2'[b,b,a,a]^T)
 * and _apply_array_spin1 (fqe_data.py:533-563: lm_apply_array1 with the
 * alpha and the beta block).  h2'[I,J,K,L] = -h2[I,K,J,L], h1' = h1 +
 * sum_K h2[I,K,K,J] over all 2 norb spin orbitals; blocks that move
 * electrons between spins do not act on a sector and are ignored.  The
 * handle works with fqegpu_apply (both precisions), fqegpu_taylor and the
 * batches; not with fqegpu_diagonal. */
int fqegpu_ham_create_spin(fqegpu_graph g, const double *h_h1,
                           const double *h_h2, void *stream, fqegpu_ham *out);
/* FQEGPU_ERR_INVALID (and nothing is freed) while a batch recorded with the
 * handle exists: destroy the batch first. */
int fqegpu_ham_destroy(fqegpu_ham h);
/* info[0] = pair count P, info[1] = 1 if compressed, info[2] = 1 if the
 * integrals are a complex scalar times a real tensor, info[3] = scratch bytes
 * of one apply at the current block width. */
int fqegpu_ham_info(fqegpu_ham h, int64_t *info4);
/* Upper bound on device scratch one apply may hold (default: 40% of free
 * memory at creation).  Smaller limits stream narrower beta-column blocks.
 * Refused (FQEGPU_ERR_INVALID) while a batch recorded with the handle exists,
 * since the batch's graph holds the current workspace. */
int fqegpu_ham_set_scratch_limit(fqegpu_ham h, int64_t bytes);

/* Tuning of the tensor-core form of this operator (no counterpart in the
 * reference): super_tiles = column tiles of 32 determinants per super-block
 * of the tile order (alpha rows inside a super-block, so psi's rows of one
 * super-block stay in L2; 0 = unchanged, default 32); use_fp64 != 0 makes
 * FQEGPU_PREC_OZAKI applies of this handle run the FP64 kernels (never less
 * accurate; cheaper for small sectors).  Chosen per sector shape by the
 * autotuner of the Python package (fqe_gb300.autotune). */
int fqegpu_ham_set_tuning(fqegpu_ham h, int super_tiles, int use_fp64);

/* Per-stage device time of the last apply on this handle (milliseconds,
 * summed over beta-column blocks): [0] gather (K2), [1] pair contraction
 * (K3), [2] scatter (K4).  Timing is measured with CUDA events recorded on
 * the launching stream when enabled with fqegpu_ham_set_timing (off by
 * default); fqegpu_ham_stage_ms waits for the last event.  No counterpart in
 * the reference (its profiling is cProfile, profiling/profile_H_ring.py). */
int fqegpu_ham_set_timing(fqegpu_ham h, int enable);
int fqegpu_ham_stage_ms(fqegpu_ham h, double *h_ms3);

/* ---- A2-A6: H·psi ---------------------------------------------------------
 * d_sigma = alpha * (H d_psi) + beta * d_psi for the sector of the graph the
 * Hamiltonian was created on.  Replaces, for one sector, FqeData.apply_inplace
 * (fqe_data.py:421-475) with its three native calls
 * lm_apply_array12_same_spin_opt x2 and lm_apply_array12_diff_spin_opt
 * (lib/fqe_data.c:668-720, :973-996; Cython wrappers _fqe_data.pyx:609-765),
 * and for one-body operators lm_apply_array1 (lib/fqe_data.c:272-302).
 * Wavefunction._apply_array's e_0 term (wavefunction.py:396-397) is beta.
 * d_psi and d_sigma must not alias.
 * Asynchronous on `stream` for both precisions (no host synchronisation), so
 * applies can be chained.  A bounded device wait of the tensor-core kernel
 * that gives up sets a sticky error word of the handle; it is reported as
 * FQEGPU_ERR_TIMEOUT by fqegpu_ham_check, or by a later apply on the handle
 * once the failed apply has finished (that later apply then does nothing). */
int fqegpu_apply(fqegpu_ham h, const double *d_psi, double *d_sigma,
                 double alpha_re, double alpha_im, double beta_re,
                 double beta_im, int precision, void *stream);
/* Waits for `stream` and reports (then clears) the handle's sticky error
 * word: FQEGPU_ERR_TIMEOUT when a tensor-core apply since the last check
 * gave up a bounded wait.  The synchronous entry points (fqegpu_apply_host,
 * fqegpu_taylor, fqegpu_batch_check) check by themselves. */
int fqegpu_ham_check(fqegpu_ham h, void *stream);
/* Same with host buffers: copies psi in and sigma out (pageable or pinned),
 * synchronous; the device staging buffer is allocated on the first call and
 * kept by the handle.  On the tensor-core path the last scatter runs in row
 * chunks and each chunk of sigma is copied out (on a copy stream the handle
 * keeps) while later chunks are scattered.  This is the call a ctypes
 * binding inside the reference's FqeData would make. */
int fqegpu_apply_host(fqegpu_ham h, const double *h_psi, double *h_sigma,
                      double alpha_re, double alpha_im, double beta_re,
                      double beta_im, int precision);

/* The same FP64 apply without any device allocation.  No counterpart in the
 * reference.  For callers that cannot allocate device memory while they run —
 * a program whose device memory belongs to another allocator (a framework's
 * caching allocator, a fixed arena) or a loop that cannot afford the device
 * synchronisation cudaMalloc/cudaFree imply.  All working memory (string
 * tables, pair matrix, D/G blocks) comes from one static 64 MiB device array
 * that every GPU loading the library holds until exit; sectors whose tables
 * plus one beta column exceed it return FQEGPU_ERR_UNSUPPORTED.  The first
 * call on a device looks up the array's address (make it before any stream
 * capture).  Calls share the array: calls that overlap on the GPU race and
 * must be serialised by the caller.  Synchronous: returns after sigma is
 * written.  h_h1 may be NULL; h_h2 is required. */
int fqegpu_apply_noalloc(int norb, int nalpha, int nbeta, const double *h_h1,
                         const double *h_h2, const double *d_psi,
                         double *d_sigma, double alpha_re, double alpha_im,
                         double beta_re, double beta_im, void *stream);

/* ---- A7: dvec ------------------------------------------------------------
 * d_dvec[i][j][a][b] = sum_J <I|E_ij|J> psi_J   (zdvec_make,
 * lib/fqe_data.c:350-377, FqeData.calculate_dvec_spatial fqe_data.py:2149)
 * and its inverse scatter d_out[I] (+)= sum_ij sum_J <I|E_ij|J> dvec_ij[J]
 * (zcoeff_make, lib/fqe_data.c:379-406, fqe_data.py:2309-2334). */
int fqegpu_make_dvec(fqegpu_graph g, const double *d_psi, double *d_dvec,
                     void *stream);
int fqegpu_make_coeff(fqegpu_graph g, const double *d_dvec, double *d_out,
                      int accumulate, void *stream);

/* ---- A11: diagonal Coulomb -------------------------------------------------
 * mode 0: d_psi[I] *= exp(E(I)) (zdiagonal_coulomb, lib/fqe_data.c:526-602)
 * mode 1: d_psi[I] *= E(I)      (zdiagonal_coulomb_apply, :455-524)
 * with E(I) = sum_{i in a} f_i + sum_{i,j in a} V_ij (same for b) plus the
 * cross term (2 V_ij rows for mode 0 as the reference, V_ij + V_ji for
 * mode 1).  h_diag complex128[norb], h_vij complex128[norb][norb], already
 * multiplied by -i t for evolution (diagonal_coulomb.py:109-123). */
int fqegpu_diagonal_coulomb(fqegpu_graph g, const double *h_diag,
                            const double *h_vij, double *d_psi, int mode,
                            void *stream);

/* ---- A13: vector operations on complex128 arrays of n elements ----------
 * FqeData.ax_plus_y / scale / norm (fqe_data.py:2620-2751), util.vdot
 * (util.py:506-530).  Results of reductions go to host memory (the call
 * synchronises on `stream`).  Reductions are deterministic. */
int fqegpu_axpy(int64_t n, double a_re, double a_im, const double *d_x,
                double *d_y, void *stream);
int fqegpu_scale(int64_t n, double a_re, double a_im, double *d_x,
                 void *stream);
int fqegpu_vdot(int64_t n, const double *d_x, const double *d_y,
                double *h_result2, void *stream);
int fqegpu_norm2(int64_t n, const double *d_x, double *h_result,
                 void *stream);
/* Block forms for a Davidson subspace (no counterpart in the reference, whose
 * Davidson works on dense numpy matrices, algorithm/davidson.py:186-268):
 *   h_out[2i..2i+1] = <V_i | t>,  i < k   (one synchronisation for all k)
 *   d_t += sum_i c_i V_i                   (one pass over d_t)
 * h_vecs: host array of k device pointers to complex128[n]; k <= 64;
 * h_coef: complex128[k] on the host.  Deterministic. */
int fqegpu_block_vdot(int64_t n, int k, const double *const *h_vecs,
                      const double *d_t, double *h_out, void *stream);
int fqegpu_block_axpy(int64_t n, int k, const double *h_coef,
                      const double *const *h_vecs, double *d_t, void *stream);

/* ---- batches of applies in one CUDA graph ----------------------------------
 * No counterpart in the reference (Wavefunction._apply_array applies sectors
 * one at a time, wavefunction.py:366-399).  Records n applies
 *   d_sigmas[i] = alpha * (H_i d_psis[i]) + beta * d_psis[i]
 * into one CUDA graph after one uncaptured pass that allocates every
 * workspace and tensor-core plan.  hams may repeat: the applies of one handle
 * run in order on one of up to eight parallel branches of the graph, and
 * applies of different handles may run concurrently, so no sigma may overlap
 * another entry's psi or sigma (FQEGPU_ERR_INVALID).
 * fqegpu_batch_launch replays the batch with one graph launch (asynchronous);
 * fqegpu_batch_check synchronises `stream` and reports a tensor-core timeout
 * of the last launch.  Buffers are those given at creation.  While a batch
 * exists its handles refuse fqegpu_ham_destroy and
 * fqegpu_ham_set_scratch_limit (the graph holds their workspaces). */
typedef struct fqegpu_batch_s *fqegpu_batch;
int fqegpu_batch_create(int n, const fqegpu_ham *hams,
                        const double *const *d_psis, double *const *d_sigmas,
                        double alpha_re, double alpha_im, double beta_re,
                        double beta_im, int precision, void *stream,
                        fqegpu_batch *out);
int fqegpu_batch_launch(fqegpu_batch b, void *stream);
int fqegpu_batch_check(fqegpu_batch b, void *stream);
int fqegpu_batch_destroy(fqegpu_batch b);
/* Taylor series of many sectors in one CUDA graph: for every i,
 *   d_psis[i] <- sum_k (-i t H_i)^k / k! d_psis[i]
 * with each sector's own stopping test (||term|| < accuracy, at most
 * expansion-1 orders; the device-resident loop of fqegpu_taylor), the sectors
 * spread over parallel branches of the graph.  No e_0 phase.  hams must be
 * distinct.  fqegpu_batch_launch runs one evolution of every sector (in
 * place, asynchronous); fqegpu_batch_taylor_terms waits, writes the number of
 * terms of each sector to h_terms[n] (may be NULL) and returns
 * FQEGPU_ERR_NUMERIC if a series did not converge.  Reference:
 * Wavefunction.apply_generated_unitary 'taylor' (wavefunction.py:553-568)
 * applied sector by sector. */
int fqegpu_batch_taylor_create(int n, const fqegpu_ham *hams,
                               double *const *d_psis, double time,
                               double accuracy, int expansion, int precision,
                               void *stream, fqegpu_batch *out);
int fqegpu_batch_taylor_terms(fqegpu_batch b, int *h_terms, void *stream);

/* ---- orbital rotation and diagonal evolution --------------------------------
 * d_psi <- (prod over icol of X^beta_icol(m_b)) (prod over icol of
 * X^alpha_icol(m_a)) d_psi, columns in ascending order, alpha first, with the
 * column operator X_icol(m) = 1 + sum_i m[i][icol] E_{i,icol} on the strings
 * of one spin: FqeData.apply_columns_recursive_inplace (fqe_data.py:1510-1535)
 * and lm_apply_array1_column_alpha (lib/fqe_data.c:305-347), the kernel of
 * Wavefunction.transform (wavefunction.py:813-959).  h_mat_a, h_mat_b:
 * complex128 [norb][norb] on the host (the host side forms them from the LU
 * factors of the rotation); d_work: a device array of the sector's size,
 * overwritten (each column is one pass from one array into the other; the
 * result ends in d_psi).  norb <= 64, at most 65535 strings per spin. */
int fqegpu_transform(fqegpu_graph g, const double *h_mat_a,
                     const double *h_mat_b, double *d_psi, double *d_work,
                     void *stream);
/* d_psi[a][b] *= exp(sum_{i in a} h_diag_a[i] + sum_{j in b} h_diag_b[j])
 * (complex128 [norb] each, already multiplied by -i t):
 * FqeData.evolve_diagonal (fqe_data.py:203-262). */
int fqegpu_evolve_diagonal(fqegpu_graph g, const double *h_diag_a,
                           const double *h_diag_b, double *d_psi,
                           void *stream);

/* ---- one-particle RDM -------------------------------------------------------
 * h_rdm[i][j] = <bra| E_ij |ket>, E_ij = sum over spin of a+_i a_j, complex128
 * [norb][norb] on the host: FqeData.rdm1(bradata) with ket = self and bra =
 * bradata (fqe_data.py:1668-1724; the blocked dvec contraction of
 * make_dvec_part, lib/fqe_data.c:604-639).  d_bra and d_ket are sector
 * coefficient arrays of the graph's sector.  D is formed on the fly, never
 * stored; deterministic; synchronises on `stream`. */
int fqegpu_rdm1(fqegpu_graph g, const double *d_bra, const double *d_ket,
                double *h_rdm, void *stream);
/* Two-particle RDM core: h_raw[kl][ij] = sum_I conj(D_bra[kl][I]) D_ket[ij][I]
 * with D[ij][I] = <I|E_ij|.> (complex128 [norb^2][norb^2] on the host), the
 * one GEMM of FqeData.rdm12's half-filling branch (fqe_data.py:1762-1781,
 * whose dvecs come from calculate_dvec_spatial); the caller assembles
 * rdm2 = -raw.reshape(n,n,n,n).transpose(1,2,0,3) plus rdm1 on the diagonal.
 * D is formed on the fly from the pair tables and never stored (no dvec of
 * norb^2 times the sector); FP64, deterministic; synchronises on `stream`.
 * When d_bra == d_ket only the upper tiles are computed (Hermitian). */
int fqegpu_rdm2_gram(fqegpu_graph g, const double *d_bra, const double *d_ket,
                     double *h_raw, void *stream);

/* ---- A10: Taylor propagator ------------------------------------------------
 * d_psi <- sum_k (-i t H)^k / k! d_psi until ||term|| < accuracy, at most
 * `expansion`-1 orders, then the e_0 phase exp(-i t e_0) (e0 passed in).
 * Wavefunction.apply_generated_unitary 'taylor' (wavefunction.py:553-568,
 * 605-606) and time_evolve's two-body branch (wavefunction.py:1042-1045).
 * *h_terms receives the number of applies.  FQEGPU_ERR_NUMERIC if the series
 * does not reach the accuracy (the reference raises RuntimeError) or a term's
 * norm is not finite.  The series runs on the device as one CUDA graph (a
 * conditional WHILE node whose body is one order: apply, accumulation, norm,
 * stopping test); the host reads the loop state once, at the end.  The graph
 * is kept by the handle and reused while the arguments stay the same.
 * Synchronous. */
int fqegpu_taylor(fqegpu_ham h, double *d_psi, double time, double e0_re,
                  double e0_im, double accuracy, int expansion, int precision,
                  int *h_terms, void *stream);

/* ---- A12: Davidson support -----------------------------------------------
 * d_diag[I] = <I|H|I> (real part, float64 [lena][lenb]) by the Slater-Condon
 * rules, in one pass (the reference builds it with one expectationValue per
 * determinant, algorithm/davidson.py:159-180). */
int fqegpu_diagonal(fqegpu_ham h, double *d_diag, void *stream);

/* Davidson correction vector, complex128[n] -> complex128[n]:
 *   d_t[I] = d_r[I] / (theta - d_diag[I]),  |theta - d_diag[I]| >= floor_
 * (the reference's diagonal preconditioner, algorithm/davidson.py:273-280,
 * where the denominator is computed on the host from the O(N) diagonal). */
int fqegpu_precondition(int64_t n, const double *d_r, const double *d_diag,
                        double theta, double floor_, double *d_t,
                        void *stream);

/* ---- A12: learned Davidson preconditioner ---------------------------------
 * No counterpart in the reference (its Davidson uses the plain diagonal
 * preconditioner, algorithm/davidson.py:273-280).  A 34 -> 64 -> 64 -> 1 MLP
 * (bfloat16 weights, float32 sums) gives each determinant a multiplier
 * m_I in (0, 2) of the diagonal preconditioner:
 *   d_t[I] = m_I d_r[I] / (theta - d_diag[I])   (|denominator| >= floor_)
 * Features: (H_II - theta) / scale, (theta - emin) / scale and the alpha and
 * beta occupations of 16 slots each, slot k holding orbital k - 8 + n_spin
 * (core slots read 1).  norb <= 16.  Parameters (float32, in this order):
 * W1[64][34], b1[64], W2[64][64], b2[64], w3[64], b3 — 6465 values.  A new
 * network has all parameters zero (m = 1: the plain preconditioner). */
typedef struct fqegpu_mlp_s *fqegpu_mlp;
int fqegpu_mlp_create(fqegpu_mlp *out);
int fqegpu_mlp_destroy(fqegpu_mlp m);
int fqegpu_mlp_nparams(void);
/* Sets the float32 master copy (and its bfloat16 image); resets Adam. */
int fqegpu_mlp_set_params(fqegpu_mlp m, const float *h_params, int64_t n);
int fqegpu_mlp_get_params(fqegpu_mlp m, float *h_params, int64_t n);
int fqegpu_mlp_get_grad(fqegpu_mlp m, float *h_grad, int64_t n);
/* Inference fused with preconditioning (complex128 r, t; float64 diag). */
int fqegpu_mlp_precondition(fqegpu_mlp m, fqegpu_graph g, const double *d_r,
                            const double *d_diag, double theta, double scale,
                            double emin, double floor_, double *d_t,
                            void *stream);
/* The multipliers alone (float32 [lena * lenb]). */
int fqegpu_mlp_multiplier(fqegpu_mlp m, fqegpu_graph g, const double *d_diag,
                          double theta, double scale, double emin, float *d_m,
                          void *stream);
/* One correction-equation sample: u = r / (theta - H_II) (floored), Ritz
 * vector x, exact correction a (a orthogonal to x), all complex128.  Loss
 *   L = 1 - |a^H v|^2 / (|a|^2 |v|^2),  v = (1 - x x^H)(m * u)
 * to *h_loss; d L / d params stored in the handle (added to the stored
 * gradient when accumulate != 0).  Synchronises on `stream`. */
int fqegpu_mlp_loss_grad(fqegpu_mlp m, fqegpu_graph g, const double *d_u,
                         const double *d_x, const double *d_a,
                         const double *d_diag, double theta, double scale,
                         double emin, int accumulate, double *h_loss,
                         void *stream);
/* Adam on the master copy with gradient * grad_scale; refreshes the bfloat16
 * weights. */
int fqegpu_mlp_adam(fqegpu_mlp m, double lr, double beta1, double beta2,
                    double eps, double grad_scale, void *stream);

/* ---- test hooks (no counterpart in the reference) --------------------------
 * Failure detection is tested without a GPU fault: the tensor-core kernel's
 * bounded waits give up after `wait_cycles` clock cycles (<= 0: the default,
 * about 2 s) and, with skip_slot >= 0, the producers of its first CTA leave
 * that ring slot of its first tile pair unfilled, so the MMA warp's wait runs
 * out and the apply reports FQEGPU_ERR_TIMEOUT (the kernel waits for the MMAs
 * it issued and frees its tensor memory before it exits).  skip_slot = -1 and
 * wait_cycles = 0 restore normal operation.  fqegpu_debug_fail_allocs makes
 * the library's next `count` device allocations fail as on an exhausted
 * device (FQEGPU_ERR_NOMEM). */
int fqegpu_ham_test_injection(fqegpu_ham h, int64_t wait_cycles, int skip_slot);
int fqegpu_debug_fail_allocs(int count);

#ifdef __cplusplus
}
#endif
#endif /* FQEGPU_H */
