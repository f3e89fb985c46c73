"""Host-side logic of the package (no GPU)."""

import numpy
import pytest


def test_alpha_beta_electrons():
    from fqe_gb300 import alpha_beta_electrons
    assert alpha_beta_electrons(14, 0) == (7, 7)
    assert alpha_beta_electrons(5, 1) == (3, 2)
    assert alpha_beta_electrons(4, -2) == (1, 3)
    with pytest.raises(ValueError):
        alpha_beta_electrons(3, 0)
    with pytest.raises(ValueError):
        alpha_beta_electrons(2, 4)
    with pytest.raises(ValueError):
        alpha_beta_electrons(-1, 0)


def test_restricted_hamiltonian_interface():
    from fqe_gb300 import RestrictedHamiltonian
    h1 = numpy.eye(3)
    h2 = numpy.zeros((3,) * 4)
    ham = RestrictedHamiltonian((h1, h2), e_0=0.5)
    assert ham.dim() == 3 and ham.rank() == 4 and not ham.quadratic()
    a, b = ham.iht(0.2)
    assert numpy.allclose(a, -0.2j * h1) and numpy.allclose(b, -0.2j * h2)
    assert RestrictedHamiltonian((h1,)).quadratic()
    with pytest.raises(ValueError):
        RestrictedHamiltonian((numpy.zeros(3),))
    with pytest.raises(TypeError):
        RestrictedHamiltonian(([1.0],))


def test_diagonal_coulomb_interface():
    from fqe_gb300 import DiagonalCoulomb
    v = numpy.arange(9.0).reshape(3, 3)
    dc = DiagonalCoulomb(v)
    assert dc.diagonal_coulomb() and numpy.all(dc._tensor[1] == 0)
    h2 = numpy.zeros((3,) * 4)
    for i in range(3):
        for j in range(3):
            h2[i, j, i, j] = -(i + 2 * j)
        h2[i, i, i, i] = 7.0 + i
    dc4 = DiagonalCoulomb(h2)
    assert numpy.allclose(dc4._tensor[1], [7, 8, 9])
    assert dc4._tensor[2][1, 2] == 1 + 4
    d, vv = dc.iht(0.1)
    assert numpy.allclose(vv, -0.1j * v)


def test_build_hamiltonian_tuple_branch():
    from fqe_gb300 import build_hamiltonian, RestrictedHamiltonian
    ham = build_hamiltonian((numpy.eye(2), numpy.zeros((2,) * 4)), norb=2)
    assert isinstance(ham, RestrictedHamiltonian)
    with pytest.raises(AssertionError):
        build_hamiltonian((numpy.zeros((2,) * 4),), norb=2)


def test_synthetic_generator_is_seeded_and_symmetric():
    from fqe_gb300 import synthetic
    h1, h2, rng = synthetic.integrals(6, 8, 0)
    h1b, h2b, _ = synthetic.integrals(6, 8, 0)
    assert numpy.array_equal(h1, h1b) and numpy.array_equal(h2, h2b)
    assert numpy.array_equal(h1, h1.T)
    # h2[i,j,k,l] = -1/2 (ik|jl) has the real-orbital pair symmetries
    assert numpy.array_equal(h2, numpy.einsum("ijkl->kjil", h2))
    assert numpy.array_equal(h2, numpy.einsum("ijkl->ilkj", h2))
    psi = synthetic.wavefunction_coeff(15, 20, rng)
    assert abs(numpy.linalg.norm(psi) - 1) < 1e-14


def test_precision_setting():
    from fqe_gb300 import settings, _lib
    assert settings.precision_code() == _lib.PREC_FP64
    settings.precision = "ozaki"
    try:
        assert settings.precision_code() == _lib.PREC_OZAKI
        settings.precision = "bogus"
        with pytest.raises(ValueError):
            settings.precision_code()
    finally:
        settings.precision = "fp64"


def test_no_cpu_fallback_without_device():
    import torch
    from fqe_gb300 import settings
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    with pytest.raises(RuntimeError):
        settings.device()


def test_rdm2_assembly_matches_reference_fixture(golden, oracle):
    # FqeData.rdm12's host-side assembly (permutation of the dvecs' Gram
    # matrix, rdm1 on the diagonal), with the Gram matrix formed here from
    # the oracle's dvecs; the device computes the same Gram matrix
    # (fqegpu_rdm2_gram, tests/test_gpu_rdm.py)
    from fqe_gb300.fqe_data import rdm2_from_gram
    gd = golden("rdm12")
    for key in [k for k in gd if k.startswith("rdm2_")]:
        tag = key[5:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        ket, bra = gd["ket_" + tag], gd["bra_" + tag]
        p = norb * norb
        dket = oracle.make_dvec(ket, g).reshape(p, -1)
        dbra = oracle.make_dvec(bra, g).reshape(p, -1)
        r1 = oracle.rdm1(ket, g)
        r2 = rdm2_from_gram(dket.conj() @ dket.T, r1)
        assert numpy.abs(r2 - gd["rdm2_" + tag]).max() < 1e-13
        t1 = oracle.rdm1(ket, g, bra)
        t2 = rdm2_from_gram(dbra.conj() @ dket.T, t1)
        assert numpy.abs(t2 - gd["trdm2_" + tag]).max() < 1e-13
