"""ORACLE — test infrastructure only (never imported by the GPU product).

A numpy model of the arithmetic of the tensor-core (FQEGPU_PREC_OZAKI) pair
contraction G = V D of this project's apply, for checking its numerical
design on the CPU.  The reference has no counterpart: it contracts in FP64
(lib/fqe_data.c:879-970); the FP64 result here is the exact reference value.

What is modelled (csrc/ozaki.cu, k_oz_digits and k_oz_fused):

* each row of V is scaled by its exponent e (max |V| < 2^e), rounded to a
  40-bit magnitude and cut into five bytes; slice a holds
  sign * byte_a * 2^-8a, exactly representable in BF16;
* psi is scaled by one global exponent g0 to a 47-bit integer and cut into
  six balanced base-256 digits in [-128, 128]; D's digit b is the signed sum
  of its (at most two) sources' digits b, in [-256, 256], exact in BF16
  (`psi_digit_slices`, `contract_psi_digits`);
* the 20 products (a, b) with a + b <= 7 (a <= 5: V slice, b <= 6: D slice)
  are summed per K step of 16 pairs into four FP32 accumulators: levels 2,
  3, 4 alone (integer sums below 2^24 at one scale: exact) and levels 5..7
  together;
* the four level sums are combined by a chain of exact two-sums (no level
  is assumed to hold the leading bits) into an unnormalised FP32 pair and
  scaled by 2^(e_row + g0 + 1).

`contract` models the form the kernel had before: D's columns scaled by
their exact exponents and rounded to 40-bit magnitudes (five slices, 19
products); it is kept to compare the two designs.  The FP32-pair scatter
that follows on the device adds about 2^-48 relative and is not modelled.
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


def _two_sum(a, b):
    s = (a + b).astype(numpy.float32)
    bb = (s - a).astype(numpy.float32)
    e = ((a - (s - bb)) + (b - bb)).astype(numpy.float32)
    return s, e


def combine_chain(acc, e_row, e_col):
    """G from the level sums by a chain of exact two-sums in FP32:
    (s, e) = two-sum(level 2, level 3), then s absorbs level 4 and levels
    5..7 the same way, the rounding errors summed in e; (s, e) is scaled by
    2^(e_row + e_col).  Unlike `combine` it does
    not assume that levels 2 and 3 hold the leading bits, which fails when
    D is scaled globally and a column's value starts in level 4 or later."""
    a = [acc[i].astype(numpy.float32) for i in range(4)]
    s, e = _two_sum(a[0], a[1])
    for k in (2, 3):
        s, e2 = _two_sum(s, a[k])
        e = (e + e2).astype(numpy.float32)
    # the pair (s, e) is stored unnormalised; the scatter's FP32-pair sum
    # takes it as it is
    scale = numpy.ldexp(1.0, e_row[:, None] + e_col[None, :])
    return (s.astype(numpy.float64) + e.astype(numpy.float64)) * scale


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


# ---- the gather-free slicing: psi cut once into digits -----------------------
# csrc/ozaki.cu, k_oz_digits / k_oz_fused: psi is scaled by one global
# exponent g0 (max |Re|, |Im| < 2^g0) to a 47-bit fixed-point integer and cut
# into six balanced base-256 digits in [-128, 128] (the last digit exact),
# stored as digit * 2^-8b; a D entry is a sum of at most two psi entries with
# signs +-1 (one alpha and one beta source), so its digit b is the sum of the
# sources' digits b, in [-256, 256]: exact in BF16, with no rounding and no
# per-column exponent.  D = 2^(g0+1) sum_b slice_b.  The 20 products a + b <= 7
# (a <= 5 slices of V, b <= 6 of D) reach 2^-48 of the global scale.

PSI_DIGITS = 6


def psi_digit_slices(psi):
    """(slices, g0): slices[b - 1] = digit_b(Re psi) 2^-8b + i digit_b(Im psi)
    2^-8b for b = 1..6, and the global exponent g0."""
    mx = max(numpy.abs(psi.real).max(), numpy.abs(psi.imag).max())
    g0 = int(numpy.frexp(mx)[1]) if mx > 0 else 0
    out = []
    parts = []
    for comp in (psi.real, psi.imag):
        x = numpy.rint(numpy.ldexp(comp, 47 - g0)).astype(numpy.int64)
        digs = []
        for b in range(1, PSI_DIGITS):
            k = 8 * (PSI_DIGITS - b)
            d = (x + (1 << (k - 1))) >> k
            x = x - (d << k)
            digs.append(d)
        digs.append(x)  # the last digit is the remainder, |x| <= 128
        parts.append(digs)
    for b in range(PSI_DIGITS):
        for d in (parts[0][b], parts[1][b]):
            assert numpy.abs(d).max() <= 128
        out.append((parts[0][b] + 1j * parts[1][b]) * 2.0 ** (-8 * (b + 1)))
    return out, g0


def digit_level_sums(vs, ds, fp32=True):
    """The four level accumulators [4, P, M] of sum_ab vs[a] ds[b] (a + b <=
    MAX_LEVEL) in K steps of 16; float64 accumulation with fp32=False."""
    dt = numpy.float32 if fp32 else numpy.float64
    P, K = vs[0].shape
    acc = numpy.zeros((4, P, ds[0].shape[1]), dtype=dt)
    for b in range(1, len(ds) + 1):
        for a in range(1, min(len(vs), MAX_LEVEL - b) + 1):
            lvl = a + b
            ai = lvl - 2 if lvl <= 4 else 3
            for k0 in range(0, K, KSTEP):
                part = vs[a - 1][:, k0:k0 + KSTEP] @ ds[b - 1][k0:k0 + KSTEP, :]
                acc[ai] = (acc[ai].astype(numpy.float64) + part).astype(dt)
    return acc


def digit_slices_of_dvec(psi, dvec):
    """D's six slices (real and imaginary columns side by side) from psi's
    digit planes through the gather dvec, and g0."""
    dslices, g0 = psi_digit_slices(psi)
    ds = []
    for b, sl in enumerate(dslices, 1):
        D = dvec(sl)
        Dr = numpy.concatenate([D.real, D.imag], axis=1)
        assert numpy.abs(Dr * 2.0 ** (8 * b)).max() <= 256
        ds.append(Dr)
    return ds, g0


def contract_psi_digits(V, psi, dvec, fp32=True):
    """The modelled tensor-core G = V D with D's slices formed from psi's
    digits: dvec(x) is the (linear, +-1) gather D = E x of the apply, applied
    to each digit plane; returns G [P, N] complex."""
    ds, g0 = digit_slices_of_dvec(psi, dvec)
    e_row = _exponents(V, 1)
    vs = slices(V, e_row[:, None])
    acc = digit_level_sums(vs, ds, fp32=fp32)
    M = ds[0].shape[1]
    e_col = numpy.full(M, g0 + 1)
    G = combine_chain(acc, e_row, e_col)
    n = M // 2
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
