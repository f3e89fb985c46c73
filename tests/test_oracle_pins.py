"""Pins the CPU oracle (oracle/) to the reference.

* against tests/golden/*.npz, produced by running the reference FQE 0.3.0
  (tests/golden/make_golden.py) — always runs;
* against the reference's own golden data (tests/unittest_data/fqe_data of
  the reference, read in place) and known-answer tests — when the reference
  tree is mounted;
* against the live reference (imported with oracle/ref_fqe.py) on extra
  seeded cases — when its natives are built in oracle/_ref.
"""

import math
import os

import numpy
import pytest

import ref_fqe

REF_DATA = os.path.join(ref_fqe.REF_ROOT, "tests", "unittest_data")


def _rel(a, b):
    return numpy.linalg.norm(a - b) / max(numpy.linalg.norm(b), 1e-300)


def test_graph_tables_match_fixture(golden, oracle):
    gd = golden("graphs")
    for key in [k for k in gd if k.startswith("astr_")]:
        tag = key[5:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        numpy.testing.assert_array_equal(g.astr, gd["astr_" + tag])
        numpy.testing.assert_array_equal(g.bstr, gd["bstr_" + tag])
        numpy.testing.assert_array_equal(g.dexca, gd["dexca_" + tag])
        numpy.testing.assert_array_equal(g.dexcb, gd["dexcb_" + tag])
        numpy.testing.assert_array_equal(g.alens.ravel(), gd["amaplen_" + tag])
        numpy.testing.assert_array_equal(g.amaps, gd["amaps_" + tag])


def test_graph_tables_match_reference_pickles(golden, oracle):
    # the reference's own stored graphs (tests/unittest_data/fci_graph/*.pickle)
    gd = golden("graph_pickles")
    tags = [k[5:] for k in gd if k.startswith("astr_")]
    assert len(tags) >= 4
    for tag in tags:
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        numpy.testing.assert_array_equal(g.astr, gd["astr_" + tag])
        numpy.testing.assert_array_equal(g.bstr, gd["bstr_" + tag])
        numpy.testing.assert_array_equal(g.dexca, gd["dexca_" + tag])
        numpy.testing.assert_array_equal(g.dexcb, gd["dexcb_" + tag])
        numpy.testing.assert_array_equal(g.alens.ravel(), gd["amaplen_" + tag])
        numpy.testing.assert_array_equal(g.amaps, gd["amaps_" + tag])


def test_string_order_known_answer(oracle):
    # tests/fci_graph_test.py:34-39 of the reference: the 70 strings of
    # (4 electrons, 8 orbitals) in address order begin 15, 23, 39, 71, 135 and
    # end 216, 232, 240; address(27) = 5, address(30) = 35.
    s = oracle.strings(8, 4)
    assert list(s[:5]) == [15, 23, 39, 71, 135]
    assert list(s[-3:]) == [216, 232, 240]
    assert list(s).index(27) == 5 and list(s).index(30) == 35
    assert len(set(s.tolist())) == 70 and all(bin(int(x)).count("1") == 4 for x in s)


def _apply_cases(gd):
    for key in [k for k in gd if k.startswith("sigma_")]:
        tag = key[6:]
        norb, na, nb = map(int, tag.split("_")[:3])
        tensors = (gd["h1_" + tag],) + ((gd["h2_" + tag],) if "h2_" + tag in gd else ())
        yield tag, norb, na, nb, tensors, gd["psi_" + tag], gd[key]


def test_apply_matches_fixture(golden, oracle):
    gd = golden("apply")
    n = 0
    for tag, norb, na, nb, tensors, psi, sigma in _apply_cases(gd):
        g = oracle.graph(norb, na, nb)
        out = oracle.apply_restricted(psi, tensors, 0.0, g)
        assert _rel(out, sigma) < 1e-13, tag
        n += 1
    assert n >= 8
    g = oracle.graph(5, 2, 2)
    out = oracle.apply_restricted(gd["e0_psi"], (gd["e0_h1"], gd["e0_h2"]), -1.25, g)
    assert _rel(out, gd["e0_sigma"]) < 1e-13


def test_diagonal_coulomb_matches_fixture(golden, oracle):
    gd = golden("diagonal_coulomb")
    for key in [k for k in gd if k.startswith("evolve_")]:
        tag = key[7:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        psi, v, f = gd["psi_" + tag], gd["v_" + tag], gd["f_" + tag]
        ev = oracle.evolve_diagonal_coulomb(psi, -1j * 0.1 * f, -1j * 0.1 * v, g)
        assert _rel(ev, gd[key]) < 1e-13
        ap = oracle.apply_diagonal_coulomb(psi, f, gd["vns_" + tag], g)
        assert _rel(ap, gd["apply_" + tag]) < 1e-13
        te = oracle.evolve_diagonal_coulomb(psi, numpy.zeros(norb, complex),
                                            -1j * 0.1 * v, g)
        assert _rel(te, gd["time_evolve_" + tag]) < 1e-13


def test_taylor_matches_fixture(golden, oracle):
    gd = golden("taylor")
    for key in [k for k in gd if k.startswith("out_")]:
        tag = key[4:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        out, _ = oracle.taylor_evolve(gd["psi_" + tag], (gd["h1_" + tag], gd["h2_" + tag]),
                                      0.0, float(gd["t_" + tag]), g,
                                      accuracy=float(gd["acc_" + tag]))
        assert _rel(out, gd[key]) < 1e-12


def test_dvec_matches_fixture(golden, oracle):
    gd = golden("dvec")
    for key in [k for k in gd if k.startswith("dvec_")]:
        tag = key[5:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        dv = oracle.make_dvec(gd["psi_" + tag], g)
        numpy.testing.assert_allclose(dv, gd[key], rtol=0, atol=1e-15)
        co = oracle.make_coeff(dv, g)
        assert _rel(co, gd["coeff_" + tag]) < 1e-14


def test_known_eigenvalue_2_body(oracle):
    # tests/fqe_data_test.py:761-827 of the reference: h2[i,j,k,l] =
    # (i+k)(j+l) * 0.02 on (2 alpha, 2 beta, 4 orbitals) has the eigenvalue
    # -7.271991091302982.  The lowest eigenvalue of H on the sector must be it.
    norb = 4
    idx = numpy.arange(norb)
    h2 = (idx[:, None, None, None] + idx[None, None, :, None]) * \
         (idx[None, :, None, None] + idx[None, None, None, :]) * 0.02
    h1 = numpy.zeros((norb, norb))
    g = oracle.graph(norb, 2, 2)
    H = oracle.dense_hamiltonian(h1, h2.astype(complex), g)
    w = numpy.linalg.eigvals(H)
    assert numpy.min(numpy.abs(w - (-7.271991091302982))) < 1e-10


def _ref_golden_available():
    return os.path.isdir(os.path.join(REF_DATA, "fqe_data"))


@pytest.mark.skipif(not _ref_golden_available(),
                    reason="reference golden data not mounted")
@pytest.mark.parametrize("na,nb,norb", [(2, 3, 6), (2, 1, 4), (1, 1, 2)])
def test_reference_golden_apply(oracle, na, nb, norb):
    # tests/unittest_data/fqe_data/{cr,ci}NNNNNN{,_1,_12} + hN files
    # (written by tests/unittest_data/fqe_data/generate_data.py)
    tag = f"{na:02d}{nb:02d}{norb:02d}"
    base = os.path.join(REF_DATA, "fqe_data")
    g = oracle.graph(norb, na, nb)
    shape = (g.lena, g.lenb)

    def cplx(stem):
        cr = numpy.fromfile(os.path.join(base, "cr" + stem + ".npy")).reshape(shape)
        ci = numpy.fromfile(os.path.join(base, "ci" + stem + ".npy")).reshape(shape)
        return cr + 1j * ci

    psi = cplx(tag)
    h1 = numpy.fromfile(os.path.join(base, f"h1{tag}.npy")).reshape((norb,) * 2)
    h2 = numpy.fromfile(os.path.join(base, f"h2{tag}.npy")).reshape((norb,) * 4)
    assert _rel(oracle.apply_spatial1(psi, h1, g), cplx(tag + "_1")) < 1e-13
    assert _rel(oracle.apply_spatial12(psi, h1 * 0, h2, g), cplx(tag + "_2")) < 1e-13
    assert _rel(oracle.apply_spatial12(psi, h1, h2, g), cplx(tag + "_12")) < 1e-13


@pytest.mark.skipif(not _ref_golden_available(),
                    reason="reference golden data not mounted")
@pytest.mark.parametrize("na,nb,norb", [(2, 3, 6), (2, 1, 4)])
def test_reference_golden_diagonal_coulomb(oracle, na, nb, norb):
    # fqe_data_test.py:268-280: evolve with dmat at t = 0.1, golden _dc
    tag = f"{na:02d}{nb:02d}{norb:02d}"
    base = os.path.join(REF_DATA, "fqe_data")
    g = oracle.graph(norb, na, nb)
    shape = (g.lena, g.lenb)

    def cplx(stem):
        cr = numpy.fromfile(os.path.join(base, "cr" + stem + ".npy")).reshape(shape)
        ci = numpy.fromfile(os.path.join(base, "ci" + stem + ".npy")).reshape(shape)
        return cr + 1j * ci

    dmat = numpy.fromfile(os.path.join(base, f"dmat{tag}.npy")).reshape(norb, norb)
    t = 0.1
    out = oracle.evolve_diagonal_coulomb(cplx(tag), numpy.zeros(norb, complex),
                                         -1j * t * dmat.astype(complex), g)
    assert _rel(out, cplx(tag + "_dc")) < 1e-13


@pytest.mark.skipif(not ref_fqe.available(), reason="reference natives not built")
def test_live_reference_random_cases(oracle):
    fqe = ref_fqe.import_fqe()
    from fqe.fqe_data import FqeData
    rng = numpy.random.default_rng(99)
    for norb, na, nb in [(3, 1, 2), (5, 3, 3), (6, 2, 4), (7, 4, 2), (8, 1, 1)]:
        h1 = rng.normal(size=(norb,) * 2) + 1j * rng.normal(size=(norb,) * 2)
        h2 = rng.normal(size=(norb,) * 4) + 1j * rng.normal(size=(norb,) * 4)
        d = FqeData(na, nb, norb)
        c = rng.normal(size=d.coeff.shape) + 1j * rng.normal(size=d.coeff.shape)
        d.coeff = c.copy()
        ref = d.apply((h1, h2)).coeff
        g = oracle.graph(norb, na, nb)
        assert _rel(oracle.apply_spatial12(c, h1, h2, g), ref) < 1e-13
        numpy.testing.assert_array_equal(g.dexca, d._core._dexca)
        numpy.testing.assert_array_equal(g.astr, d._core._astr)


def test_davidson_known_answers_dense(golden, oracle):
    # The oracle's dense H (unit-vector applies) reproduces the two energies
    # the reference's tests assert: LiH ground state -8.877719570384043
    # (tests/davidson_test.py:27, with build_lih_data's integrals) and the
    # four-fold degenerate -7.271991091302982 of fqe_data_test.py:766.
    gd = golden("davidson")
    g = oracle.graph(6, 2, 2)
    H = oracle.dense_hamiltonian(gd["lih_h1"].astype(complex),
                                 gd["lih_h2"].astype(complex), g)
    w = numpy.linalg.eigvalsh(0.5 * (H + H.conj().T))
    assert abs(w[0] - float(gd["lih_e_test"])) < 1e-10
    psi = gd["lih_ground"].ravel()
    assert abs(numpy.vdot(psi, H @ psi) - gd["lih_e_expectation"]) < 1e-12
    assert abs(float(gd["lih_e_ref_davidson"][0]) - w[0]) < 1e-8
    g4 = oracle.graph(4, 2, 2)
    H4 = oracle.dense_hamiltonian(gd["k4_h1"], gd["k4_h2"], g4)
    w4 = numpy.linalg.eigvalsh(0.5 * (H4 + H4.conj().T))
    assert numpy.allclose(w4[:4], float(gd["k4_e_test"]), atol=1e-12)
    # the reference Davidson's eigenvalue-change rule stops above the exact root
    assert 1e-6 < gd["k4_e_ref_davidson"][0] - w4[0] < 1e-3


def test_rdm1_matches_fixture(golden, oracle):
    # FqeData.rdm1 of the reference, both code paths and a transition RDM
    gd = golden("rdm")
    for key in [k for k in gd if k.startswith("rdm1_")]:
        tag = key[5:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        r = oracle.rdm1(gd["ket_" + tag], g)
        assert numpy.abs(r - gd["rdm1_" + tag]).max() < 1e-14
        assert numpy.abs(r - gd["rdm1py_" + tag]).max() < 1e-14
        t = oracle.rdm1(gd["ket_" + tag], g, gd["bra_" + tag])
        assert numpy.abs(t - gd["trdm1_" + tag]).max() < 1e-14
        assert abs(numpy.trace(r) - (na + nb)) < 1e-12  # normalised ket


def test_rdm12_matches_fixture(golden, oracle):
    # FqeData.rdm12 of the reference: half-filling branch (blocked and plain)
    # and low-filling python branch, with and without a bra.  Two reference
    # quirks limit what is pinned for transition RDMs: the low-filling C
    # branch ("c" keys: an FqeData made with the accelerated switch off,
    # called with it on) forms the bra's same-spin intermediates from the
    # ket's coefficients (fqe_data.py:1958-1963, 2000-2009 pass self.coeff),
    # and both low-filling branches return rdm1(bradata), whose
    # non-accelerated form ignores the bra (fqe_data.py:1721-1724).
    gd = golden("rdm12")
    for key in [k for k in gd if k.startswith("rdm2_")]:
        tag = key[5:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        r1, r2 = oracle.rdm12(gd["ket_" + tag], g)
        t1, t2 = oracle.rdm12(gd["ket_" + tag], g, gd["bra_" + tag])
        for sfx in ("", "py", "c"):
            assert numpy.abs(r1 - gd[f"rdm1{sfx}_{tag}"]).max() < 1e-13
            assert numpy.abs(r2 - gd[f"rdm2{sfx}_{tag}"]).max() < 1e-13
        assert numpy.abs(t1 - gd[f"trdm1_{tag}"]).max() < 1e-13
        for sfx in ("", "py"):
            assert numpy.abs(t2 - gd[f"trdm2{sfx}_{tag}"]).max() < 1e-13
        # rdm2[a, b, c, d] = <sum_st a+_as a+_bt a_cs a_dt>, so contracting b
        # with d gives -(N - 1) rdm1[a, c]
        ne = na + nb
        assert numpy.abs(numpy.einsum("ikjk->ij", r2) + (ne - 1) * r1).max() < 1e-12


def test_spin_orbital_apply_matches_fixture(golden, oracle):
    # FqeData.apply with spin-orbital (2n-dimensional) one- and two-body
    # operators, the reference's own outputs
    gd = golden("spin")
    for key in [k for k in gd if k.startswith("spin12_")]:
        tag = key[7:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        psi, h1, h2 = gd["psi_" + tag], gd["h1_" + tag], gd["h2_" + tag]
        out1 = oracle.apply_spin1(psi, h1, g)
        assert numpy.abs(out1 - gd["spin1_" + tag]).max() < 1e-12
        out12 = oracle.apply_spin12(psi, h1, h2, g)
        scale = max(1.0, numpy.abs(gd[key]).max())
        assert numpy.abs(out12 - gd[key]).max() < 1e-12 * scale
    # a spin-free operator written in spin orbitals is the spatial apply
    norb, na, nb = 4, 2, 1
    g = oracle.graph(norb, na, nb)
    rng = numpy.random.default_rng(3)
    h1 = rng.normal(size=(norb, norb))
    h2 = rng.normal(size=(norb,) * 4)
    psi = rng.normal(size=(g.lena, g.lenb)) + 0j
    H1 = numpy.kron(numpy.eye(2), h1)
    H2 = numpy.zeros((2 * norb,) * 4)
    for s in (slice(0, norb), slice(norb, 2 * norb)):
        for t in (slice(0, norb), slice(norb, 2 * norb)):
            H2[s, t, s, t] = h2
    want = oracle.apply_spatial12(psi, h1, h2, g)
    assert numpy.abs(oracle.apply_spin12(psi, H1, H2, g) - want).max() < 1e-12


def test_reference_wavefunction_pickles(golden, oracle):
    # the reference's own Wavefunction.apply golden data
    # (tests/unittest_data/wavefunction/*.pickle, wavefunction_test.py:609-627),
    # unpacked by tests/golden/make_golden.py: restricted Hamiltonians
    # ('apply_array') and diagonal Coulomb ('apply_dc'), every sector
    gd = golden("wfn_pickles")
    n = 0
    for key in [k for k in gd if k.startswith("out_")]:
        name, kind, na, nb = key[4:].rsplit("_", 3)
        tag = f"{name}_{kind}"
        norb = int(gd["norb_" + tag])
        g = oracle.graph(norb, int(na), int(nb))
        psi = gd[f"psi_{tag}_{na}_{nb}"]
        e0 = complex(gd["e0_" + tag])
        if kind == "array":
            out = oracle.apply_restricted(psi, (gd["t0_" + tag], gd["t1_" + tag]), e0, g)
        else:
            out = oracle.apply_diagonal_coulomb(psi, gd["diag_" + tag], gd["vij_" + tag], g)
            if abs(e0) > 1e-15:
                out = out + e0 * psi
        want = gd[key]
        assert numpy.abs(out - want).max() <= 1e-12 * max(1.0, numpy.abs(want).max())
        n += 1
    assert n >= 15


def test_orbital_transform_matches_fixture(golden, oracle):
    # Wavefunction.transform of the reference (wavefunction.py:813-959): with
    # P L U = U^H (scipy's LU of the rotation's adjoint, P returned), the
    # sector is mapped by M = P^T U^H — here through compound matrices, an
    # independent route to the reference's recursive column operators
    gd = golden("transform")
    n = 0
    for key in [k for k in gd if k.startswith("out_")]:
        tag = key[4:]
        norb, na, nb, _ = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        U, P = gd["rot_" + tag], gd["perm_" + tag]
        M = P.T @ U.conj().T
        if U.shape[0] == norb:
            ma = mb = M
        else:
            ma, mb = M[:norb, :norb], M[norb:, norb:]
        out = oracle.transform_orbitals(gd["psi_" + tag], ma, mb, g)
        assert numpy.abs(out - gd[key]).max() < 1e-12
        n += 1
    assert n == 5


def test_chebyshev_matches_fixture(golden, oracle):
    # apply_generated_unitary(..., 'chebyshev', ...) of the reference
    gd = golden("chebyshev")
    for key in [k for k in gd if k.startswith("out_")]:
        tag = key[4:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        out = oracle.chebyshev_evolve(gd["psi_" + tag], (gd["h1_" + tag], gd["h2_" + tag]),
                                      complex(gd["e0_" + tag]), float(gd["t_" + tag]), g,
                                      list(gd["lim_" + tag]), accuracy=1e-13,
                                      expansion=200)
        assert numpy.abs(out - gd[key]).max() < 1e-12
        # unitary but for e_0's imaginary part, whose phase the reference
        # applies twice (inside H and again at the end)
        e0, t = complex(gd["e0_" + tag]), float(gd["t_" + tag])
        assert abs(numpy.linalg.norm(out) - numpy.exp(2 * t * e0.imag)) < 1e-11


def test_orbital_transform_is_a_representation(oracle):
    # compound matrices compose (Cauchy-Binet: C(M1 M2) = C(M1) C(M2)) and a
    # unitary orbital rotation keeps the sector's norm
    from scipy.stats import unitary_group
    norb, na, nb = 5, 2, 3
    g = oracle.graph(norb, na, nb)
    U1 = unitary_group.rvs(norb, random_state=7)
    U2 = unitary_group.rvs(norb, random_state=8)
    rng = numpy.random.default_rng(9)
    psi = rng.normal(size=(g.lena, g.lenb)) + 1j * rng.normal(size=(g.lena, g.lenb))
    both = oracle.transform_orbitals(psi, U1 @ U2, U1 @ U2, g)
    step = oracle.transform_orbitals(oracle.transform_orbitals(psi, U2, U2, g), U1, U1, g)
    assert numpy.abs(both - step).max() < 1e-12
    assert abs(numpy.linalg.norm(both) - numpy.linalg.norm(psi)) < 1e-12
