"""One- and two-particle RDMs (FqeData.rdm1, fqe_data.py:1668-1724;
FqeData.rdm12, :1726-1838) on the GPU against the reference's own outputs
(tests/golden/rdm.npz, rdm12.npz) and the oracle."""

import numpy
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _data(gpu, norb, na, nb, c):
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data", raw_data=c)
    return d


def test_rdm1_matches_reference(gpu, golden):
    gd = golden("rdm")
    for key in [k for k in gd if k.startswith("rdm1_")]:
        tag = key[5:]
        norb, na, nb = map(int, tag.split("_"))
        ket = _data(gpu, norb, na, nb, gd["ket_" + tag])
        bra = _data(gpu, norb, na, nb, gd["bra_" + tag])
        numpy.testing.assert_allclose(ket.rdm1()[0], gd["rdm1_" + tag],
                                      atol=TOL, rtol=0)
        numpy.testing.assert_allclose(ket.rdm1(bra)[0], gd["trdm1_" + tag],
                                      atol=TOL, rtol=0)


@pytest.mark.parametrize("norb,na,nb", [(8, 4, 3), (10, 5, 5), (7, 0, 3),
                                        (12, 6, 6)])
def test_rdm1_vs_oracle(gpu, oracle, norb, na, nb):
    from fqe_gb300 import synthetic
    _, _, psi = synthetic.sector(norb, na, nb, 2 * norb, seed=norb)
    rng = numpy.random.default_rng(norb)
    bra_c = synthetic.wavefunction_coeff(psi.shape[0], psi.shape[1], rng)
    g = oracle.graph(norb, na, nb)
    ket = _data(gpu, norb, na, nb, psi)
    bra = _data(gpu, norb, na, nb, bra_c)
    r = ket.rdm1()[0]
    want = oracle.rdm1(psi, g)
    numpy.testing.assert_allclose(r, want, atol=TOL, rtol=0)
    assert abs(numpy.trace(r) - (na + nb)) < 1e-11   # particle number
    numpy.testing.assert_allclose(r, r.conj().T, atol=TOL, rtol=0)  # Hermitian
    numpy.testing.assert_allclose(ket.rdm1(bra)[0], oracle.rdm1(psi, g, bra_c),
                                  atol=TOL, rtol=0)
    # deterministic
    assert numpy.array_equal(ket.rdm1()[0], r)


def test_rdm1_sector_mismatch(gpu):
    a = gpu.FqeData(2, 2, 4)
    b = gpu.FqeData(2, 1, 4)
    with pytest.raises(ValueError):
        a.rdm1(b)


def test_rdm12_matches_reference(gpu, golden):
    # FqeData.rdm12 (fqe_data.py:1726-1838) against the reference's
    # half-filling branch, with and without a bra (tests/golden/rdm12.npz)
    gd = golden("rdm12")
    for key in [k for k in gd if k.startswith("rdm2_")]:
        tag = key[5:]
        norb, na, nb = map(int, tag.split("_"))
        ket = _data(gpu, norb, na, nb, gd["ket_" + tag])
        bra = _data(gpu, norb, na, nb, gd["bra_" + tag])
        r1, r2 = ket.rdm12()
        numpy.testing.assert_allclose(r1, gd["rdm1_" + tag], atol=TOL, rtol=0)
        numpy.testing.assert_allclose(r2, gd["rdm2_" + tag], atol=TOL, rtol=0)
        t1, t2 = ket.rdm12(bra)
        numpy.testing.assert_allclose(t1, gd["trdm1_" + tag], atol=TOL, rtol=0)
        numpy.testing.assert_allclose(t2, gd["trdm2_" + tag], atol=TOL, rtol=0)
    with pytest.raises(ValueError):
        gpu.FqeData(2, 2, 4).rdm12(gpu.FqeData(2, 1, 4))


@pytest.mark.parametrize("norb,na,nb", [(8, 4, 3), (10, 5, 5)])
def test_rdm2_gram_vs_oracle_dvecs(gpu, oracle, norb, na, nb):
    # the dvecs' Gram matrix formed on the fly on the device against the
    # oracle's explicit dvecs (calculate_dvec_spatial), with and without a
    # distinct bra
    from fqe_gb300 import synthetic
    from fqe_gb300.fqe_data import rdm2_from_gram
    _, _, ket = synthetic.sector(norb, na, nb, 2 * norb, seed=1)
    _, _, bra = synthetic.sector(norb, na, nb, 2 * norb, seed=2)
    g = oracle.graph(norb, na, nb)
    p = norb * norb
    dk = oracle.make_dvec(ket, g).reshape(p, -1)
    db = oracle.make_dvec(bra, g).reshape(p, -1)
    k = gpu.FqeData(na, nb, norb)
    k.set_wfn(strategy="from_data", raw_data=ket)
    b = gpu.FqeData(na, nb, norb)
    b.set_wfn(strategy="from_data", raw_data=bra)
    r1, r2 = k.rdm12()
    want = rdm2_from_gram(dk.conj() @ dk.T, oracle.rdm1(ket, g))
    assert numpy.abs(r2 - want).max() < 1e-12 * max(1.0, numpy.abs(want).max())
    t1, t2 = k.rdm12(b)
    want_t = rdm2_from_gram(db.conj() @ dk.T, oracle.rdm1(ket, g, bra))
    assert numpy.abs(t2 - want_t).max() < 1e-12 * max(1.0, numpy.abs(want_t).max())


def test_rdm2_headline_sector(gpu):
    # norb 14 (7a,7b), 11.8 M determinants: no dvec of 196 x 11.8 M is formed;
    # the Hermitian shortcut (bra is ket) agrees with the general form (bra a
    # copy), and the result is Hermitian
    import time
    import torch
    from fqe_gb300 import synthetic
    _, _, psi = synthetic.sector(14, 7, 7, 28, seed=0)
    k = gpu.FqeData(7, 7, 14)
    k.set_wfn(strategy="from_data", raw_data=psi)
    copy_ = gpu.FqeData(7, 7, 14)
    copy_.coeff.copy_(k.coeff)
    torch.cuda.synchronize()
    t0 = time.time()
    r1, r2 = k.rdm12()
    t1 = time.time()
    _, r2b = k.rdm12(copy_)
    print(f"norb 14 rdm12: {t1 - t0:.2f} s (Hermitian tiles)")
    scale = numpy.abs(r2).max()
    assert numpy.abs(r2 - r2b).max() < 1e-13 * scale
    assert numpy.abs(r2b - r2b.transpose(3, 2, 1, 0).conj()).max() < 1e-13 * scale
    assert abs(numpy.trace(r1) - 14.0) < 1e-10
