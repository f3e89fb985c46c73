"""Orbital rotation (Wavefunction.transform, wavefunction.py:813-959, with
the column operators of FqeData.apply_columns_recursive_inplace on the GPU)
and the quadratic branch of time evolution (wavefunction.py:1008-1032),
against the reference's own outputs (tests/golden/transform.npz,
tests/golden/quadratic.npz) and the oracle."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


def test_transform_matches_reference(gpu, golden):
    gd = golden("transform")
    for key in [k for k in gd if k.startswith("out_")]:
        tag = key[4:]
        norb, na, nb, _ = map(int, tag.split("_"))
        w = gpu.Wavefunction([[na + nb, na - nb, norb]])
        w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): gd["psi_" + tag]})
        perm, low, upp, res = w.transform(gd["rot_" + tag])
        assert numpy.array_equal(perm, gd["perm_" + tag])
        got = res.get_coeff((na + nb, na - nb)).cpu().numpy()
        assert numpy.abs(got - gd[key]).max() < 1e-12
        assert numpy.linalg.norm(got) == pytest.approx(
            numpy.linalg.norm(gd["psi_" + tag]), abs=1e-12)


def test_transform_larger_sector(gpu, oracle):
    # norb 8 (4a,3b): the oracle's independent route (compound matrices of
    # M = P^T U^H) to the same rotation
    from scipy.stats import unitary_group
    from fqe_gb300 import synthetic
    norb, na, nb = 8, 4, 3
    _, _, psi = synthetic.sector(norb, na, nb, 16, seed=4)
    U = unitary_group.rvs(norb, random_state=7)
    w = gpu.Wavefunction([[na + nb, na - nb, norb]])
    w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi})
    perm, _, _, res = w.transform(U)
    got = res.get_coeff((na + nb, na - nb)).cpu().numpy()
    M = perm.T @ U.conj().T
    want = oracle.transform_orbitals(psi, M, M, oracle.graph(norb, na, nb))
    assert numpy.abs(got - want).max() < 1e-11
    assert numpy.linalg.norm(got) == pytest.approx(1.0, abs=1e-12)


def test_quadratic_time_evolution_matches_reference(gpu, golden):
    gd = golden("quadratic")
    for key in [k for k in gd if k.startswith("out_")]:
        tag = key[4:]
        norb, na, nb, _ = map(int, tag.split("_"))
        w = gpu.Wavefunction([[na + nb, na - nb, norb]])
        w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): gd["psi_" + tag]})
        ham = gpu.get_restricted_hamiltonian((gd["h1_" + tag],),
                                             e_0=complex(gd["e0_" + tag]))
        res = w.time_evolve(float(gd["t_" + tag]), ham)
        got = res.get_coeff((na + nb, na - nb)).cpu().numpy()
        assert numpy.abs(got - gd[key]).max() < 1e-12


def test_evolve_diagonal(gpu, oracle):
    from fqe_gb300 import synthetic
    norb, na, nb = 6, 3, 2
    _, _, psi = synthetic.sector(norb, na, nb, 12, seed=9)
    g = oracle.graph(norb, na, nb)
    rng = numpy.random.default_rng(3)
    arr = -1j * 0.3 * (rng.normal(size=2 * norb) + 0.1j * rng.normal(size=2 * norb))
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data", raw_data=psi)
    got = d.evolve_diagonal(arr).cpu().numpy()
    ea = numpy.array([sum(arr[i] for i in range(norb) if int(s) >> i & 1) for s in g.astr])
    eb = numpy.array([sum(arr[norb + i] for i in range(norb) if int(s) >> i & 1)
                      for s in g.bstr])
    want = psi * numpy.exp(ea[:, None] + eb[None, :])
    assert numpy.abs(got - want).max() < 1e-14
