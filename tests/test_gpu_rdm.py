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
