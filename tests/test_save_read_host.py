"""The on-disk form of a wavefunction (Wavefunction.save / read,
wavefunction.py:726-765), host side: a file written by the reference's own
Wavefunction.save (tests/golden/ref_saved_wfn.pickle, made by
tests/golden/make_golden.py) is decoded without the reference package into
its records and the sectors' coefficients."""

import os

import numpy

from conftest import GOLDEN


def test_reference_file_decodes(golden):
    from fqe_gb300.wavefunction import load_records, sector_arrays
    want = golden("saved_wfn")
    with open(os.path.join(GOLDEN, "ref_saved_wfn.pickle"), "rb") as fh:
        data = load_records(fh)
    sym, conserved, cspin, cnum, norb = data[:5]
    assert sym == {} and cnum and norb == 4
    assert conserved["n"] == 4
    keys = []
    for key, sector in data[5:]:
        na, nb, n, coeff = sector_arrays(sector)
        assert n == 4 and na + nb == key[0] and na - nb == key[1]
        assert numpy.array_equal(coeff, want[f"coeff_{key[0]}_{key[1]}"])
        keys.append(tuple(key))
    assert sorted(keys) == [(4, -2), (4, 0), (4, 2)]


def test_lu_regrouping_reproduces_the_rotation():
    # the host side of Wavefunction.transform: rotation^H = P L U, and the
    # regrouped factors (unit lower)^H (upper)^H give back L U
    from scipy.stats import unitary_group
    from fqe_gb300.wavefunction import column_factors, lu_factors
    U = unitary_group.rvs(6, random_state=3)
    P, L, Uu = lu_factors(U)
    assert numpy.allclose(P @ L @ Uu, U.T.conj())
    lowt, uppt = column_factors(L, Uu)
    assert numpy.allclose(numpy.triu(lowt, 1), 0.0)
    assert numpy.allclose(numpy.diag(lowt), 1.0)
    assert numpy.allclose(numpy.tril(uppt, -1), 0.0)
    assert numpy.allclose((lowt @ uppt).T.conj(), L @ Uu)
