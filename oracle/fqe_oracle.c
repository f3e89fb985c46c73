/*
 * ORACLE — test infrastructure only.  Not part of the GPU product.
 *
 * A CPU restatement, in plain C99 + OpenMP, of the reference OpenFermion-FQE
 * natives that lie on the restricted H·psi path.  It is used
 *   - by tests/ as the reference the CUDA library's results are compared with
 *     (never as the thing tested),
 *   - by bench.py's `cpu_baseline` leg and `--impl reference` arm as the timed
 *     CPU implementation of the reference algorithm (same loop structure as the
 *     reference: per-target sparse accumulation for the same-spin terms and the
 *     per-orbital-pair gather for the opposite-spin term).
 * Parity of this restatement is pinned against the reference itself (compiled
 * from its sources into oracle/_ref) and against the reference's own golden
 * data, by tests/test_oracle_pins.py and the fixtures in tests/golden/.
 *
 * Conventions (all from the reference):
 *   strings   uint64 bit masks, bit p = orbital p occupied; address order is the
 *             Knowles-Handy lexicographic order given by the Z matrix.
 *   maps      for each (i, j), i-major, a list of (source, target, sign) with
 *             <target| a+_i a_j |source> = sign.
 *   dexc      per target string, nele*(norb-nele+1) rows (source, i*norb+j, sign)
 *             in the order the maps are visited.
 *   coeff     complex128 [lena][lenb], alpha-major.
 */
#include <complex.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex zc;

#define ORC_OK 0
#define ORC_EINVAL 1
#define ORC_ENOMEM 2

/* y[k] += w * x[k] on interleaved complex doubles; the role of BLAS zaxpy in
 * the reference (passed in from SciPy, lib/_blas_helpers.h:21-36). */
static inline void orc_zaxpy(int n, zc w, const zc *restrict x, zc *restrict y) {
  const double wr = creal(w), wi = cimag(w);
  const double *restrict xs = (const double *)x;
  double *restrict ys = (double *)y;
  for (int k = 0; k < n; ++k) {
    const double xr = xs[2 * k], xi = xs[2 * k + 1];
    ys[2 * k] += wr * xr - wi * xi;
    ys[2 * k + 1] += wr * xi + wi * xr;
  }
}

static int64_t orc_binom(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  if (k > n - k) k = n - k;
  int64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int64_t orc_binomial(int n, int k) { return orc_binom(n, k); }

/* Knowles-Handy addressing matrix, Z[k][l] for the k-th electron (0-based) on
 * orbital l.  Follows lib/fci_graph.c:27-54 (and fci_graph.py:66-96). */
int orc_z_matrix(int norb, int nele, int32_t *Z) {
  if (norb < 0 || nele < 0 || nele > norb || norb > 63) return ORC_EINVAL;
  memset(Z, 0, sizeof(int32_t) * (size_t)nele * (size_t)norb);
  for (int k = 1; k < nele; ++k) {
    for (int l = k; l <= norb - nele + k; ++l) {
      int64_t acc = 0;
      for (int m = norb - l + 1; m <= norb - k; ++m)
        acc += orc_binom(m, nele - k) - orc_binom(m - 1, nele - k - 1);
      Z[(k - 1) * norb + (l - 1)] = (int32_t)acc;
    }
  }
  if (nele > 0)
    for (int l = nele; l <= norb; ++l) Z[(nele - 1) * norb + (l - 1)] = l - nele;
  return ORC_OK;
}

/* Address of a string: sum over its occupied orbitals (ascending) of Z[k][occ_k]
 * (lib/fci_graph.c:123-134). */
static int orc_index(uint64_t s, const int32_t *Z, int norb) {
  int idx = 0, k = 0;
  while (s) {
    int p = __builtin_ctzll(s);
    idx += Z[k * norb + p];
    ++k;
    s &= s - 1;
  }
  return idx;
}

int orc_string_index(uint64_t s, const int32_t *Z, int norb) {
  return orc_index(s, Z, norb);
}

/* All C(norb, nele) strings, stored at their address
 * (lib/bitstring.c:29-45 generator, lib/fci_graph.c:136-147 placement). */
int orc_strings(int norb, int nele, const int32_t *Z, uint64_t *out) {
  if (norb < 0 || nele < 0 || nele > norb || norb > 63) return ORC_EINVAL;
  if (nele == 0) {
    out[0] = 0;
    return ORC_OK;
  }
  uint64_t c = (nele == 64) ? ~0ull : ((1ull << nele) - 1);
  const uint64_t lim = 1ull << norb;
  while (c < lim) {
    out[orc_index(c, Z, norb)] = c;
    /* next combination with the same popcount, in increasing integer order */
    const uint64_t low = c & (~c + 1);
    const uint64_t ripple = c + low;
    c = (((ripple ^ c) >> 2) / low) | ripple;
  }
  return ORC_OK;
}

/* Parity of the occupied orbitals strictly between i and j
 * (lib/bitstring.h:66-71). */
static int orc_sign_between(uint64_t s, int i, int j) {
  int lo = i < j ? i : j, hi = i < j ? j : i;
  if (hi - lo < 2) return 1;
  uint64_t mask = ((1ull << hi) - 1) & ~((2ull << lo) - 1);
  return (__builtin_popcountll(s & mask) & 1) ? -1 : 1;
}

/* Lengths of the norb*norb excitation maps (lib/fci_graph.c:76-121, count
 * pass).  lengths[i*norb+j]. */
int orc_map_lengths(int norb, int len, const uint64_t *strings, int32_t *lengths) {
  for (int i = 0; i < norb; ++i)
    for (int j = 0; j < norb; ++j) {
      int cnt = 0;
      for (int s = 0; s < len; ++s) {
        const uint64_t st = strings[s];
        if (i == j) {
          if (st >> i & 1ull) ++cnt;
        } else if ((st >> j & 1ull) && !(st >> i & 1ull)) {
          ++cnt;
        }
      }
      lengths[i * norb + j] = cnt;
    }
  return ORC_OK;
}

/* Fill the maps (fill pass): maps is the concatenation, in i-major order, of
 * lengths[i*norb+j] rows of (source, target, sign). */
int orc_build_maps(int norb, int nele, int len, const uint64_t *strings,
                   const int32_t *Z, int32_t *maps) {
  (void)nele;
  int32_t *row = maps;
  for (int i = 0; i < norb; ++i)
    for (int j = 0; j < norb; ++j)
      for (int s = 0; s < len; ++s) {
        const uint64_t st = strings[s];
        if (i == j) {
          if (st >> i & 1ull) {
            row[0] = s; row[1] = s; row[2] = 1;
            row += 3;
          }
        } else if ((st >> j & 1ull) && !(st >> i & 1ull)) {
          const uint64_t t = (st & ~(1ull << j)) | (1ull << i);
          row[0] = s;
          row[1] = orc_index(t, Z, norb);
          row[2] = orc_sign_between(st, i, j);
          row += 3;
        }
      }
  return ORC_OK;
}

/* De-excitation lists from the maps (fci_graph.py:36-63, lib/fci_graph.c:57-73):
 * dexc[target][k] = (source, i*norb+j, sign), k counting per target in map
 * order. */
int orc_dexc(int norb, int nele, int len, const int32_t *lengths,
             const int32_t *maps, int32_t *dexc) {
  const int lk = nele * (norb - nele + 1);
  int *fill = calloc((size_t)len + 1, sizeof(int));
  if (!fill) return ORC_ENOMEM;
  const int32_t *row = maps;
  for (int ij = 0; ij < norb * norb; ++ij)
    for (int e = 0; e < lengths[ij]; ++e, row += 3) {
      const int tgt = row[1];
      if (fill[tgt] >= lk) { free(fill); return ORC_EINVAL; }
      int32_t *d = dexc + 3 * ((size_t)tgt * lk + fill[tgt]);
      d[0] = row[0]; d[1] = ij; d[2] = row[2];
      fill[tgt] += 1;
    }
  free(fill);
  return ORC_OK;
}

/* Same-spin part, sigma += (sum h1 E + sum h2 E E) on one spin, following the
 * reference's per-target sparse accumulation (lib/fqe_data.c:668-720).  For
 * is_alpha the "states1" index runs over rows of coeff, otherwise over
 * columns.  h1 [norb*norb], h2 [norb^2 * norb^2] are the prepared tensors
 * (h1', h2' of fqe_data.py:691-693). */
static int orc_same_spin_rows(const zc *coeff, zc *out, const int32_t *dexc,
                              int n1, int n2, int ndexc, const zc *h1,
                              const zc *h2, int norb);

int orc_apply12_same_spin(const zc *coeff, zc *out, const int32_t *dexc,
                          int lena, int lenb, int ndexc, const zc *h1,
                          const zc *h2, int norb, int is_alpha) {
  if (is_alpha)
    return orc_same_spin_rows(coeff, out, dexc, lena, lenb, ndexc, h1, h2, norb);
  /* beta: work on the transpose, as the reference's wrapper does
   * (_fqe_data.pyx:679-680, fqe_data.py:698-701) */
  const size_t n = (size_t)lena * lenb;
  zc *ct = malloc(sizeof(zc) * (n ? n : 1));
  zc *ot = calloc(n ? n : 1, sizeof(zc));
  if (!ct || !ot) { free(ct); free(ot); return ORC_ENOMEM; }
#pragma omp parallel for schedule(static)
  for (int a = 0; a < lena; ++a)
    for (int b = 0; b < lenb; ++b) ct[(size_t)b * lena + a] = coeff[(size_t)a * lenb + b];
  const int rc = orc_same_spin_rows(ct, ot, dexc, lenb, lena, ndexc, h1, h2, norb);
#pragma omp parallel for schedule(static)
  for (int a = 0; a < lena; ++a)
    for (int b = 0; b < lenb; ++b) out[(size_t)a * lenb + b] += ot[(size_t)b * lena + a];
  free(ct);
  free(ot);
  return rc;
}

static int orc_same_spin_rows(const zc *coeff, zc *out, const int32_t *dexc,
                              int n1, int n2, int ndexc, const zc *h1,
                              const zc *h2, int norb) {
  const size_t st1 = (size_t)n2;
  const int norb2 = norb * norb;
  int err = 0;
#pragma omp parallel
  {
    zc *acc = malloc(sizeof(zc) * (size_t)(n1 > 0 ? n1 : 1));
    if (!acc) {
#pragma omp atomic write
      err = 1;
    }
#pragma omp for schedule(dynamic, 1)
    for (int t = 0; t < n1; ++t) {
      if (!acc) continue;
      for (int s = 0; s < n1; ++s) acc[s] = 0;
      const int32_t *d1 = dexc + 3 * (size_t)t * ndexc;
      for (int a = 0; a < ndexc; ++a) {
        const int mid = d1[3 * a], ij = d1[3 * a + 1], p1 = d1[3 * a + 2];
        acc[mid] += p1 * h1[ij];
        const int32_t *d2 = dexc + 3 * (size_t)mid * ndexc;
        const zc *h2row = h2 + (size_t)ij * norb2;
        for (int b = 0; b < ndexc; ++b)
          acc[d2[3 * b]] += (p1 * d2[3 * b + 2]) * h2row[d2[3 * b + 1]];
      }
      zc *o = out + (size_t)t * st1;
      for (int s = 0; s < n1; ++s) {
        const zc w = acc[s];
        if (w == 0) continue;
        orc_zaxpy(n2, w, coeff + (size_t)s * st1, o);
      }
    }
    free(acc);
  }
  return err ? ORC_ENOMEM : ORC_OK;
}

/* Opposite-spin part, sigma += sum_{ij,kl} h2ab[ij,kl] E^a_ij E^b_kl coeff,
 * following the reference's loop over alpha orbital pairs with a gathered
 * block of rows (lib/fqe_data.c:879-970).  h2ab = h2' + h2'^T (pair swap). */
int orc_apply12_diff_spin(const zc *coeff, zc *out, const int32_t *adexc,
                          const int32_t *bdexc, int lena, int lenb, int nadexc,
                          int nbdexc, const zc *h2ab, int norb) {
  const int norb2 = norb * norb;
  int maxsig = 0;
  int *cnt = calloc((size_t)norb2, sizeof(int));
  if (!cnt) return ORC_ENOMEM;
  for (size_t e = 0; e < (size_t)lena * nadexc; ++e) cnt[adexc[3 * e + 1]] += 1;
  for (int p = 0; p < norb2; ++p) maxsig = cnt[p] > maxsig ? cnt[p] : maxsig;
  free(cnt);
  int *tgt = malloc(sizeof(int) * (size_t)(maxsig + 1));
  int *src = malloc(sizeof(int) * (size_t)(maxsig + 1));
  int *sgn = malloc(sizeof(int) * (size_t)(maxsig + 1));
  zc *blk = malloc(sizeof(zc) * ((size_t)maxsig * lenb + 1));
  if (!tgt || !src || !sgn || !blk) {
    free(tgt); free(src); free(sgn); free(blk);
    return ORC_ENOMEM;
  }
  int err = 0;
  for (int ij = 0; ij < norb2; ++ij) {
    int nsig = 0;
    for (int a = 0; a < lena; ++a)
      for (int e = 0; e < nadexc; ++e) {
        const int32_t *d = adexc + 3 * ((size_t)a * nadexc + e);
        if (d[1] == ij) {
          tgt[nsig] = a; src[nsig] = d[0]; sgn[nsig] = d[2];
          ++nsig;
        }
      }
    if (!nsig) continue;
    /* blk[jb][q] = sign_q * coeff[src_q][jb] */
#pragma omp parallel for schedule(static)
    for (int jb = 0; jb < lenb; ++jb)
      for (int q = 0; q < nsig; ++q)
        blk[(size_t)jb * nsig + q] = sgn[q] * coeff[(size_t)src[q] * lenb + jb];
    const zc *hrow = h2ab + (size_t)ij * norb2;
#pragma omp parallel
    {
      zc *v = malloc(sizeof(zc) * (size_t)nsig);
      if (!v) {
#pragma omp atomic write
        err = 1;
      }
#pragma omp for schedule(static)
      for (int b = 0; b < lenb; ++b) {
        if (!v) continue;
        for (int q = 0; q < nsig; ++q) v[q] = 0;
        for (int e = 0; e < nbdexc; ++e) {
          const int32_t *d = bdexc + 3 * ((size_t)b * nbdexc + e);
          orc_zaxpy(nsig, d[2] * hrow[d[1]], blk + (size_t)d[0] * nsig, v);
        }
        for (int q = 0; q < nsig; ++q) out[(size_t)tgt[q] * lenb + b] += v[q];
      }
      free(v);
    }
  }
  free(tgt); free(src); free(sgn); free(blk);
  return err ? ORC_ENOMEM : ORC_OK;
}

/* One-body part on one spin (lib/fqe_data.c:272-302): out[t] += sum over
 * dexc[t] of sign * h1[ij] * coeff[source]. */
int orc_apply1(const zc *coeff, zc *out, const int32_t *dexc, int lena,
               int lenb, int ndexc, const zc *h1, int is_alpha) {
  const int n1 = is_alpha ? lena : lenb;
  const int n2 = is_alpha ? lenb : lena;
  const size_t st1 = is_alpha ? (size_t)lenb : 1;
  const size_t st2 = is_alpha ? 1 : (size_t)lenb;
#pragma omp parallel for schedule(static)
  for (int t = 0; t < n1; ++t) {
    zc *o = out + (size_t)t * st1;
    for (int e = 0; e < ndexc; ++e) {
      const int32_t *d = dexc + 3 * ((size_t)t * ndexc + e);
      const zc w = d[2] * h1[d[1]];
      const zc *c = coeff + (size_t)d[0] * st1;
      for (int k = 0; k < n2; ++k) o[k * st2] += w * c[k * st2];
    }
  }
  return ORC_OK;
}

static int orc_occ(uint64_t s, int *occ) {
  int n = 0;
  while (s) {
    occ[n++] = __builtin_ctzll(s);
    s &= s - 1;
  }
  return n;
}

/* Diagonal-Coulomb evolution (lib/fqe_data.c:526-602): with f = exp(diag),
 * V = exp(array) elementwise,
 *   coeff[a][b] *= (prod_{i in a, j in b} V[i][j])^2 * A[a] * B[b],
 *   A[s] = prod_{i in s} f[i] * prod_{i,j in s} V[i][j]. */
int orc_diagonal_coulomb(const uint64_t *astr, const uint64_t *bstr,
                         const zc *diag, const zc *array, zc *coeff, int lena,
                         int lenb, int norb) {
  zc *fexp = malloc(sizeof(zc) * (size_t)norb);
  zc *vexp = malloc(sizeof(zc) * (size_t)norb * norb);
  zc *ad = malloc(sizeof(zc) * (size_t)lena);
  zc *bd = malloc(sizeof(zc) * (size_t)lenb);
  if (!fexp || !vexp || !ad || !bd) {
    free(fexp); free(vexp); free(ad); free(bd);
    return ORC_ENOMEM;
  }
  for (int i = 0; i < norb; ++i) fexp[i] = cexp(diag[i]);
  for (int i = 0; i < norb * norb; ++i) vexp[i] = cexp(array[i]);
  for (int pass = 0; pass < 2; ++pass) {
    const uint64_t *str = pass ? bstr : astr;
    zc *dst = pass ? bd : ad;
    const int len = pass ? lenb : lena;
    for (int s = 0; s < len; ++s) {
      int occ[64];
      const int n = orc_occ(str[s], occ);
      zc p = 1;
      for (int x = 0; x < n; ++x) {
        p *= fexp[occ[x]];
        for (int y = 0; y < n; ++y) p *= vexp[occ[x] * norb + occ[y]];
      }
      dst[s] = p;
    }
  }
#pragma omp parallel for schedule(static)
  for (int a = 0; a < lena; ++a) {
    int occ[64];
    zc row[64];
    const int n = orc_occ(astr[a], occ);
    for (int i = 0; i < norb; ++i) row[i] = 1;
    for (int x = 0; x < n; ++x)
      for (int i = 0; i < norb; ++i) row[i] *= vexp[occ[x] * norb + i];
    for (int b = 0; b < lenb; ++b) {
      int bocc[64];
      const int m = orc_occ(bstr[b], bocc);
      zc p = 1;
      for (int y = 0; y < m; ++y) p *= row[bocc[y]];
      coeff[(size_t)a * lenb + b] *= p * p * bd[b] * ad[a];
    }
  }
  free(fexp); free(vexp); free(ad); free(bd);
  return ORC_OK;
}

/* Diagonal-Coulomb apply (lib/fqe_data.c:455-524):
 *   coeff[a][b] *= sum_{i in a, j in b} (V[i][j] + V[j][i]) + A[a] + B[b],
 *   A[s] = sum_{i in s} f[i] + sum_{i,j in s} V[i][j]. */
int orc_diagonal_coulomb_apply(const uint64_t *astr, const uint64_t *bstr,
                               const zc *diag, const zc *array, zc *coeff,
                               int lena, int lenb, int norb) {
  zc *ad = malloc(sizeof(zc) * (size_t)lena);
  zc *bd = malloc(sizeof(zc) * (size_t)lenb);
  if (!ad || !bd) {
    free(ad); free(bd);
    return ORC_ENOMEM;
  }
  for (int pass = 0; pass < 2; ++pass) {
    const uint64_t *str = pass ? bstr : astr;
    zc *dst = pass ? bd : ad;
    const int len = pass ? lenb : lena;
    for (int s = 0; s < len; ++s) {
      int occ[64];
      const int n = orc_occ(str[s], occ);
      zc p = 0;
      for (int x = 0; x < n; ++x) {
        p += diag[occ[x]];
        for (int y = 0; y < n; ++y) p += array[occ[x] * norb + occ[y]];
      }
      dst[s] = p;
    }
  }
#pragma omp parallel for schedule(static)
  for (int a = 0; a < lena; ++a) {
    int occ[64];
    zc row[64];
    const int n = orc_occ(astr[a], occ);
    for (int i = 0; i < norb; ++i) row[i] = 0;
    for (int x = 0; x < n; ++x)
      for (int i = 0; i < norb; ++i)
        row[i] += array[occ[x] * norb + i] + array[i * norb + occ[x]];
    for (int b = 0; b < lenb; ++b) {
      int bocc[64];
      const int m = orc_occ(bstr[b], bocc);
      zc p = 0;
      for (int y = 0; y < m; ++y) p += row[bocc[y]];
      coeff[(size_t)a * lenb + b] *= p + bd[b] + ad[a];
    }
  }
  free(ad); free(bd);
  return ORC_OK;
}

/* dvec[ij] += E_ij coeff for one spin, from the maps (lib/fqe_data.c:350-377).
 * dvec is [norb*norb][lena][lenb]; maps/lengths as produced above. */
int orc_make_dvec(const int32_t *lengths, const int32_t *maps, int norb,
                  const zc *coeff, zc *dvec, int lena, int lenb, int is_alpha) {
  const size_t plane = (size_t)lena * lenb;
  size_t *off = malloc(sizeof(size_t) * ((size_t)norb * norb + 1));
  if (!off) return ORC_ENOMEM;
  off[0] = 0;
  for (int ij = 0; ij < norb * norb; ++ij) off[ij + 1] = off[ij] + lengths[ij];
#pragma omp parallel for schedule(dynamic)
  for (int ij = 0; ij < norb * norb; ++ij) {
    zc *d = dvec + (size_t)ij * plane;
    for (size_t e = off[ij]; e < off[ij + 1]; ++e) {
      const int s = maps[3 * e], t = maps[3 * e + 1], p = maps[3 * e + 2];
      if (is_alpha) {
        for (int b = 0; b < lenb; ++b)
          d[(size_t)t * lenb + b] += p * coeff[(size_t)s * lenb + b];
      } else {
        for (int a = 0; a < lena; ++a)
          d[(size_t)a * lenb + t] += p * coeff[(size_t)a * lenb + s];
      }
    }
  }
  free(off);
  return ORC_OK;
}

/* coeff[I] += sum_ij sum_J <I|E_ij|J> dvec[ij][J] for one spin
 * (lib/fqe_data.c:379-406, driven as fqe_data.py:2309-2334).  The reference
 * visits map (j, i) and adds dvec[ij] at that map's target into its source;
 * since <t|E_ji|s> = <s|E_ij|t>, this is the same as: for every entry
 * (s, t, p) of map (i, j), i.e. <t|E_ij|s> = p, coeff[t] += p * dvec[ij][s]. */
int orc_make_coeff(const int32_t *lengths, const int32_t *maps, int norb,
                   zc *coeff, const zc *dvec, int lena, int lenb, int is_alpha) {
  const size_t plane = (size_t)lena * lenb;
  const int32_t *row = maps;
  for (int ij = 0; ij < norb * norb; ++ij) {
    const zc *d = dvec + (size_t)ij * plane;
    for (int e = 0; e < lengths[ij]; ++e, row += 3) {
      const int s = row[0], t = row[1], p = row[2];
      if (is_alpha) {
        for (int b = 0; b < lenb; ++b)
          coeff[(size_t)t * lenb + b] += p * d[(size_t)s * lenb + b];
      } else {
        for (int a = 0; a < lena; ++a)
          coeff[(size_t)a * lenb + t] += p * d[(size_t)a * lenb + s];
      }
    }
  }
  return ORC_OK;
}
