"""ORACLE — test infrastructure only (never imported by the GPU product).

A numpy model of the arithmetic of the tensor-core (FQEGPU_PREC_OZAKI) pair
contraction G = V D of this project's apply, for checking its numerical
design on the CPU.  The reference has no counterpart: it contracts in FP64
(lib/fqe_data.c:879-970); the FP64 result here is the exact reference value.

What is modelled (csrc/ozaki.cu, k_oz_slice / k_oz_mma):

* each real column of D (one determinant, real or imaginary part, all pair
  rows) is scaled by its exact exponent e (max |D| < 2^e) and rounded to a
  40-bit magnitude; each row of V likewise with its row exponent;
* a 40-bit magnitude m is cut into five bytes; slice k holds
  sign * byte_k * 2^-8k, exactly representable in BF16;
* the 19 products (a, b) with a + b <= 7 (a: V slice, b: D slice) are summed
  per K step of 16 pairs into four FP32 accumulators: levels 2, 3, 4 alone
  (integer sums below 2^24 at one scale: exact) and levels 5..7 together;
* the four level sums are combined by an exact two-sum of levels 2 and 3,
  the low part adding levels 4 and 5..7, and scaled by 2^(e_row + e_col).

The determinant-side exponents here come straight from D (the kernel
derives them from a 62-bit fixed-point copy of psi, which adds at most
2^-62 relative); the FP32-pair scatter that follows on the device adds about
2^-48 relative and is not modelled.
"""

import numpy

SLICES = 5
BITS = 8
MAX_LEVEL = 7
KSTEP = 16


def _exponents(x, axis):
    """e with max |x| < 2^e along `axis` (frexp convention; 0 for all-zero)."""
    mx = numpy.abs(x).max(axis=axis)
    return numpy.frexp(mx)[1]


def slices(x, e):
    """Five slices of x (real) against the exponents e (broadcast to x): the
    40-bit rounded magnitude m = round(|x| 2^(40-e)) cut into bytes, slice k
    = sign * byte_k * 2^-8k."""
    tot = SLICES * BITS
    m = numpy.minimum(numpy.floor(numpy.abs(x) * numpy.ldexp(1.0, tot - e) + 0.5),
                      2.0 ** tot - 1.0)
    sgn = numpy.sign(x)
    out = []
    for k in range(1, SLICES + 1):
        byte = numpy.floor(m / 2.0 ** (tot - BITS * k)) % 2 ** BITS
        out.append(sgn * byte * 2.0 ** (-BITS * k))
    return out


def level_sums(V, D, fp32=True, e_col=None):
    """The four level accumulators of G = V D for real V [P, K], D [K, M]:
    returns (acc [4, P, M], e_row [P], e_col [M]).  With fp32=False the
    accumulation runs in float64 (to show where FP32 rounds); `e_col`
    replaces the exact column exponents by given upper bounds."""
    e_row = _exponents(V, 1)
    if e_col is None:
        e_col = _exponents(D, 0)
    vs = slices(V, e_row[:, None])
    ds = slices(D, e_col[None, :])
    dt = numpy.float32 if fp32 else numpy.float64
    P, K = V.shape
    acc = numpy.zeros((4, P, D.shape[1]), dtype=dt)
    for b in range(1, SLICES + 1):
        for a in range(1, min(SLICES, MAX_LEVEL - b) + 1):
            lvl = a + b
            ai = lvl - 2 if lvl <= 4 else 3
            for k0 in range(0, K, KSTEP):
                part = vs[a - 1][:, k0:k0 + KSTEP] @ ds[b - 1][k0:k0 + KSTEP, :]
                acc[ai] = (acc[ai].astype(numpy.float64) + part).astype(dt)
    return acc, e_row, e_col


def combine(acc, e_row, e_col):
    """G from the level sums: (h, l) = two-sum(level 2, level 3), l += level 4
    + levels 5..7 (FP32), then (h + l) scaled by 2^(e_row + e_col), returned
    as float64 of the FP32 pair."""
    x = acc[0].astype(numpy.float32)
    y = acc[1].astype(numpy.float32)
    h = (x + y).astype(numpy.float32)
    bb = (h - x).astype(numpy.float32)
    l = ((x - (h - bb)) + (y - bb)).astype(numpy.float32)
    l = (l + acc[2].astype(numpy.float32)).astype(numpy.float32)
    l = (l + acc[3].astype(numpy.float32)).astype(numpy.float32)
    h2 = (h + l).astype(numpy.float32)
    l2 = (l - (h2 - h)).astype(numpy.float32)
    scale = numpy.ldexp(1.0, e_row[:, None] + e_col[None, :])
    return (h2.astype(numpy.float64) + l2.astype(numpy.float64)) * scale


def psi_bound_exponents(psi):
    """Per-determinant exponent bounds from psi alone: every D[q][a, b] is a
    sum of at most one psi entry of column b (alpha source) and one of row a
    (beta source), so |D| < 2^(max(rowexp(a), colexp(b)) + 1)."""
    ex = numpy.frexp(numpy.maximum(numpy.abs(psi.real), numpy.abs(psi.imag)))[1]
    eb = numpy.maximum(ex.max(axis=1)[:, None], ex.max(axis=0)[None, :]) + 1
    return eb.ravel()


def contract(V, D, e_det=None):
    """The modelled tensor-core G = V D for real V [P, K] and complex D [K, N]
    (real and imaginary columns side by side, as on the device).  `e_det`
    [N] replaces the exact per-column exponents by per-determinant bounds
    (for both the real and the imaginary column)."""
    Dr = numpy.concatenate([D.real, D.imag], axis=1)
    e_col = None if e_det is None else numpy.concatenate([e_det, e_det])
    acc, e_row, e_col = level_sums(V, Dr, e_col=e_col)
    G = combine(acc, e_row, e_col)
    n = D.shape[1]
    return G[:, :n] + 1j * G[:, n:]


def pair_matrix(h1, h2, nele, prep):
    """V[ij][kl] = h2'[i,j,k,l] + h1'[i,j] delta_kl / N_e (uncompressed pairs)
    from the reference's h1'/h2' preparation `prep` (fqe_data.py:691-693)."""
    h1p, h2p = prep(h1, h2)
    n = h1p.shape[0]
    V = h2p.reshape(n * n, n * n).copy()
    for ij in range(n * n):
        for k in range(n):
            V[ij, k * n + k] += h1p.reshape(-1)[ij] / nele
    return V
