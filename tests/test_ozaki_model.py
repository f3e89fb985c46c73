"""The numerical design of the tensor-core (Ozaki-split BF16) contraction,
checked on the CPU with the numpy model oracle/ozaki_model.py: V in five
8-bit slices of 40-bit fixed point per row, psi cut once into six balanced
8-bit digits at one global exponent (D's digits are exact sums of two
sources' digits), 20 products a + b <= 7, four FP32 level accumulators,
two-sum combination.  The level sums 2-4 are exact, and the contraction and
the apply stay within the 1e-10 relative bound the GPU tests hold the kernel
to, for spread-out and for concentrated psi.  The earlier per-column form
(exact column exponents, five D slices) is compared alongside.  The same
design's device results are compared with the oracle in
tests/test_gpu_ozaki.py."""

import numpy
import pytest


def _rel(a, b):
    return numpy.linalg.norm(a - b) / numpy.linalg.norm(b)


def _case(oracle, norb, na, nb, seed, peaked=False):
    import ozaki_model as om
    from fqe_gb300 import synthetic
    h1, h2, psi = synthetic.sector(norb, na, nb, 2 * norb, seed)
    if peaked:
        rng = numpy.random.default_rng(seed)
        psi = 1e-6 * (rng.normal(size=psi.shape) + 1j * rng.normal(size=psi.shape))
        psi[0, 0] = 0.99
        psi[-1, 1] = -0.1j
    g = oracle.graph(norb, na, nb)
    V = om.pair_matrix(h1, h2, na + nb, oracle.prep_spatial12)
    assert numpy.abs(V.imag).max() == 0.0  # real integrals: the tensor-core form
    D = oracle.make_dvec(psi, g).reshape(norb * norb, -1)
    return h1, h2, psi, g, V.real.copy(), D


def _dvec(oracle, g, norb):
    return lambda x: oracle.make_dvec(x, g).reshape(norb * norb, -1)


def test_psi_digits_reconstruct_psi():
    import ozaki_model as om
    rng = numpy.random.default_rng(2)
    psi = rng.normal(size=(40, 30)) + 1j * rng.normal(size=(40, 30))
    psi[3, 4] = 7.5 - 0.25j
    sl, g0 = om.psi_digit_slices(psi)
    back = 2.0 ** (g0 + 1) * sum(sl)
    # 47-bit fixed point at the global scale: |error| <= 2^(g0 - 48) in the
    # real and in the imaginary part
    assert numpy.abs((back - psi).real).max() <= 2.0 ** (g0 - 48)
    assert numpy.abs((back - psi).imag).max() <= 2.0 ** (g0 - 48)
    for b, x in enumerate(sl, 1):
        for part in (x.real, x.imag):
            d = part * 2.0 ** (8 * b)
            assert numpy.array_equal(d, numpy.round(d))  # integers
            assert numpy.abs(d).max() <= 128


def test_digit_levels_2_to_4_are_exact(oracle):
    import ozaki_model as om
    *_, g, V, _ = _case(oracle, 8, 4, 4, 3)
    _, _, psi = __import__("fqe_gb300.synthetic", fromlist=["x"]).sector(8, 4, 4, 16, 3)
    ds, _ = om.digit_slices_of_dvec(psi, _dvec(oracle, g, 8))
    vs = om.slices(V, om._exponents(V, 1)[:, None])
    a32 = om.digit_level_sums(vs, ds, fp32=True)
    a64 = om.digit_level_sums(vs, ds, fp32=False)
    for lvl in range(3):  # levels 2, 3, 4
        assert numpy.array_equal(a32[lvl].astype(numpy.float64), a64[lvl])
    assert numpy.abs(a32[3] - a64[3]).max() <= 2.0 ** -40 * numpy.abs(a64[0]).max()


@pytest.mark.parametrize("norb,na,nb,peaked", [(8, 4, 4, False), (8, 3, 5, False),
                                               (10, 5, 5, False), (8, 4, 4, True),
                                               (10, 5, 5, True)])
def test_digit_contraction_and_apply_within_bound(oracle, norb, na, nb, peaked):
    import ozaki_model as om
    h1, h2, psi, g, V, D = _case(oracle, norb, na, nb, norb + na, peaked)
    G = om.contract_psi_digits(V, psi, _dvec(oracle, g, norb))
    assert _rel(G, V @ D) < 3e-11  # measured 3e-12 (spread) to 1e-11 (peaked)
    shape = (norb, norb, g.lena, g.lenb)
    ref = oracle.apply_spatial12(psi, h1, h2, g)
    # measured 2.4e-12 to 7.7e-12: well inside the 1e-10 bound
    assert _rel(oracle.make_coeff(G.reshape(shape), g), ref) < 2e-11


def test_levels_2_to_4_are_exact(oracle):
    import ozaki_model as om
    *_, V, D = _case(oracle, 8, 4, 4, 3)
    Dr = numpy.concatenate([D.real, D.imag], axis=1)
    a32, _, _ = om.level_sums(V, Dr, fp32=True)
    a64, _, _ = om.level_sums(V, Dr, fp32=False)
    for lvl in range(3):  # levels 2, 3, 4
        assert numpy.array_equal(a32[lvl].astype(numpy.float64), a64[lvl])
    # levels 5..7 share one accumulator and round, far below level 2's scale
    assert numpy.abs(a32[3] - a64[3]).max() <= 2.0 ** -40 * numpy.abs(a64[0]).max()


@pytest.mark.parametrize("norb,na,nb,peaked", [(8, 4, 4, False), (8, 3, 5, False),
                                               (10, 3, 3, False), (8, 4, 4, True)])
def test_contraction_and_apply_within_bound(oracle, norb, na, nb, peaked):
    import ozaki_model as om
    h1, h2, psi, g, V, D = _case(oracle, norb, na, nb, norb + na, peaked)
    G64 = V @ D
    G = om.contract(V, D)
    assert _rel(G, G64) < 1e-11  # measured 2-3e-12
    shape = (norb, norb, g.lena, g.lenb)
    ref = oracle.apply_spatial12(psi, h1, h2, g)
    # the FP64 dvec form is the reference's apply ...
    assert _rel(oracle.make_coeff(G64.reshape(shape), g), ref) < 1e-12
    # ... and the modelled tensor-core contraction stays well within the
    # 1e-10 bound (measured 3-4e-12, as the kernel on the GPU)
    assert _rel(oracle.make_coeff(G.reshape(shape), g), ref) < 1e-11


@pytest.mark.parametrize("peaked", [False, True])
def test_exponents_bounded_from_psi(oracle, peaked):
    # the cheaper choice for a kernel that slices while it contracts:
    # exponents bounded from psi's row and column maxima instead of the exact
    # column maxima of D cost a factor 2-3 in error (measured 5e-12 to
    # 1e-11), still an order of magnitude inside the 1e-10 bound
    import ozaki_model as om
    h1, h2, psi, g, V, D = _case(oracle, 8, 4, 4, 11, peaked)
    ref = oracle.apply_spatial12(psi, h1, h2, g)
    G = om.contract(V, D, e_det=om.psi_bound_exponents(psi))
    sigma = oracle.make_coeff(G.reshape(8, 8, g.lena, g.lenb), g)
    assert _rel(sigma, ref) < 3e-11


def test_fewer_slices_would_break_the_bound(oracle):
    # the design's margin: stopping the products at level 5 instead of 7
    # leaves an error far above 1e-10
    import ozaki_model as om
    *_, V, D = _case(oracle, 8, 4, 4, 5)
    Dr = numpy.concatenate([D.real, D.imag], axis=1)
    old = om.MAX_LEVEL
    try:
        om.MAX_LEVEL = 5
        acc, er, ec = om.level_sums(V, Dr)
        G5 = om.combine(acc, er, ec)
    finally:
        om.MAX_LEVEL = old
    assert _rel(G5, V @ Dr) > 1e-9


def test_digit_form_on_taylor_terms(oracle):
    # the high-order terms of a Taylor series are more concentrated than a
    # random psi; at one global scale their small columns start in level 4
    # or later, where a combination that assumes levels 2-3 lead loses bits
    # (1e-11 per apply, measured): the two-sum chain keeps them at ~5e-13
    import ozaki_model as om
    from fqe_gb300 import synthetic
    norb, na, nb = 10, 5, 5
    h1, h2, psi = synthetic.sector(norb, na, nb, 20, 4)
    g = oracle.graph(norb, na, nb)
    V = om.pair_matrix(h1, h2, na + nb, oracle.prep_spatial12).real.copy()
    w = psi.copy()
    for _ in range(18):
        w = oracle.apply_spatial12(w, h1, h2, g)
        w /= numpy.linalg.norm(w)
    dv = _dvec(oracle, g, norb)
    D = dv(w)
    shape = (norb, norb, g.lena, g.lenb)
    ref = oracle.make_coeff((V @ D).reshape(shape), g)
    G = om.contract_psi_digits(V, w, dv)
    assert _rel(oracle.make_coeff(G.reshape(shape), g), ref) < 2e-12
    ds, g0 = om.digit_slices_of_dvec(w, dv)
    vs = om.slices(V, om._exponents(V, 1)[:, None])
    acc = om.digit_level_sums(vs, ds)
    e_row = om._exponents(V, 1)
    e_col = numpy.full(ds[0].shape[1], g0 + 1)
    naive = om.combine(acc, e_row, e_col)
    n = naive.shape[1] // 2
    Gn = naive[:, :n] + 1j * naive[:, n:]
    assert _rel(oracle.make_coeff(Gn.reshape(shape), g), ref) > 5e-12


def test_digit_form_needs_level_7(oracle):
    # with psi's digits at one global exponent, dropping level 7 (15 instead
    # of 20 products) leaves psi effectively 40-bit at the global scale: too
    # coarse for a concentrated psi
    import ozaki_model as om
    h1, h2, psi, g, V, D = _case(oracle, 10, 5, 5, 15, True)
    old = om.MAX_LEVEL
    try:
        om.MAX_LEVEL = 6
        G6 = om.contract_psi_digits(V, psi, _dvec(oracle, g, 10))
    finally:
        om.MAX_LEVEL = old
    G7 = om.contract_psi_digits(V, psi, _dvec(oracle, g, 10))
    assert _rel(G6, V @ D) > 5 * _rel(G7, V @ D)
