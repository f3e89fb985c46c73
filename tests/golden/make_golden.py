"""Generate tests/golden/*.npz by running the reference FQE (0.3.0).

Run in a container where the reference sources are mounted and
``make -C oracle ref`` has built its natives:

    python tests/golden/make_golden.py

Every fixture records the reference's own output for seeded inputs; the GPU
tests and the oracle pin tests compare against these files, so nothing at test
time needs the reference.  Inputs come from fqe_gb300.synthetic (a numpy-only
module) or from numpy.random.default_rng with the seeds written below.
"""

import math
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "openfermion-fqe_gb300"))

import ref_fqe  # noqa: E402
from fqe_gb300 import synthetic  # noqa: E402  (numpy only)

fqe = ref_fqe.import_fqe()
from fqe.fqe_data import FqeData  # noqa: E402
from fqe.fci_graph import FciGraph  # noqa: E402

GRAPH_CASES = [(4, 2, 2), (6, 3, 2), (8, 4, 4), (5, 0, 3), (3, 3, 1),
               (7, 2, 5), (1, 1, 0), (10, 5, 4)]
APPLY_CASES = [  # (norb, nalpha, nbeta, kind, seed)
    (4, 2, 2, "real", 1),
    (6, 3, 2, "real", 2),
    (8, 4, 4, "real", 0),
    (5, 2, 3, "complex", 3),
    (6, 1, 4, "nonsym", 4),
    (7, 3, 3, "real", 5),
    (4, 0, 2, "real", 6),
    (6, 3, 3, "onebody", 7),
    (5, 2, 2, "onebody_complex", 8),
]


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    numpy.savez_compressed(path, **arrays)
    print("wrote", path, sum(a.nbytes for a in arrays.values()), "bytes raw")


def graph_fixture():
    out = {}
    for norb, na, nb in GRAPH_CASES:
        g = FciGraph(na, nb, norb)
        tag = f"{norb}_{na}_{nb}"
        out[f"astr_{tag}"] = numpy.asarray(g._astr, dtype=numpy.uint64)
        out[f"bstr_{tag}"] = numpy.asarray(g._bstr, dtype=numpy.uint64)
        out[f"dexca_{tag}"] = numpy.asarray(g._dexca, dtype=numpy.int32)
        out[f"dexcb_{tag}"] = numpy.asarray(g._dexcb, dtype=numpy.int32)
        maps = [numpy.asarray(g._alpha_map[(i, j)], dtype=numpy.int32).reshape(-1, 3)
                for i in range(norb) for j in range(norb)]
        out[f"amaplen_{tag}"] = numpy.array([len(m) for m in maps], dtype=numpy.int32)
        out[f"amaps_{tag}"] = (numpy.concatenate(maps) if maps else
                               numpy.zeros((0, 3), numpy.int32))
    save("graphs", **out)


def graph_pickles_fixture():
    """The reference's own stored FciGraph objects
    (tests/unittest_data/fci_graph/NNAANBNO.pickle, checked by
    tests/fci_graph_test.py), unpacked into the tables of graph_fixture."""
    import pickle
    src = os.path.join(ref_fqe.REF_ROOT, "tests", "unittest_data", "fci_graph")
    out = {}
    for f in sorted(os.listdir(src)):
        if not f.endswith(".pickle"):
            continue
        with open(os.path.join(src, f), "rb") as fh:
            g = pickle.load(fh)["graph"]
        norb, na, nb = g._norb, g._nalpha, g._nbeta
        tag = f"{norb}_{na}_{nb}"
        out[f"astr_{tag}"] = numpy.asarray(g._astr, dtype=numpy.uint64)
        out[f"bstr_{tag}"] = numpy.asarray(g._bstr, dtype=numpy.uint64)
        out[f"dexca_{tag}"] = numpy.asarray(g._dexca, dtype=numpy.int32)
        out[f"dexcb_{tag}"] = numpy.asarray(g._dexcb, dtype=numpy.int32)
        maps = [numpy.asarray(g._alpha_map[(i, j)], dtype=numpy.int32).reshape(-1, 3)
                for i in range(norb) for j in range(norb)]
        out[f"amaplen_{tag}"] = numpy.array([len(m) for m in maps], dtype=numpy.int32)
        out[f"amaps_{tag}"] = (numpy.concatenate(maps) if maps else
                               numpy.zeros((0, 3), numpy.int32))
    save("graph_pickles", **out)


def make_tensors(norb, kind, seed):
    rng = numpy.random.default_rng(1000 + seed)
    if kind == "real":
        h1, h2, _ = synthetic.integrals(norb, 2 * norb, seed)
        return h1, h2
    if kind in ("complex", "nonsym"):
        h1 = rng.normal(size=(norb, norb)) + 1j * rng.normal(size=(norb, norb))
        h2 = (rng.normal(size=(norb,) * 4) + 1j * rng.normal(size=(norb,) * 4)) * 0.3
        if kind == "complex":  # hermitian h1, h2 with the hermitian pair symmetry
            h1 = 0.5 * (h1 + h1.conj().T)
            h2 = 0.5 * (h2 + numpy.einsum("ijkl->lkji", h2.conj()))
        return h1, h2
    if kind == "onebody":
        h1 = rng.normal(size=(norb, norb))
        return (0.5 * (h1 + h1.T),)
    if kind == "onebody_complex":
        return (rng.normal(size=(norb, norb)) + 1j * rng.normal(size=(norb, norb)),)
    raise ValueError(kind)


def apply_fixture():
    out = {}
    for norb, na, nb, kind, seed in APPLY_CASES:
        tensors = make_tensors(norb, kind, seed)
        d = FqeData(na, nb, norb)
        rng = numpy.random.default_rng(2000 + seed)
        c = synthetic.wavefunction_coeff(d.lena(), d.lenb(), rng)
        d.coeff = c.copy()
        res = d.apply(tensors).coeff
        tag = f"{norb}_{na}_{nb}_{kind}"
        out[f"psi_{tag}"] = c
        out[f"h1_{tag}"] = numpy.asarray(tensors[0], dtype=numpy.complex128)
        if len(tensors) > 1:
            out[f"h2_{tag}"] = numpy.asarray(tensors[1], dtype=numpy.complex128)
        out[f"sigma_{tag}"] = numpy.asarray(res)
    # Wavefunction.apply with e_0 (wavefunction.py:396-397)
    norb, na, nb = 5, 2, 2
    h1, h2, _ = synthetic.integrals(norb, 10, 11)
    wfn = fqe.Wavefunction([[na + nb, na - nb, norb]])
    rng = numpy.random.default_rng(2011)
    c = synthetic.wavefunction_coeff(math.comb(norb, na), math.comb(norb, nb), rng)
    wfn.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): c})
    ham = fqe.get_restricted_hamiltonian((h1, h2), e_0=-1.25)
    res = wfn.apply(ham)
    out["e0_psi"] = c
    out["e0_h1"] = h1
    out["e0_h2"] = h2
    out["e0_sigma"] = res.get_coeff((na + nb, na - nb))
    save("apply", **out)


def dc_fixture():
    out = {}
    for norb, na, nb, seed in [(6, 3, 2, 0), (8, 4, 4, 1), (5, 0, 2, 2)]:
        v = synthetic.diagonal_coulomb(norb, seed)
        rng = numpy.random.default_rng(3000 + seed)
        vns = rng.normal(size=(norb, norb))  # non-symmetric for the apply
        f = rng.normal(size=norb)
        d = FqeData(na, nb, norb)
        c = synthetic.wavefunction_coeff(d.lena(), d.lenb(), rng)
        tag = f"{norb}_{na}_{nb}"
        t = 0.1
        d.coeff = c.copy()
        ev = d.evolve_diagonal_coulomb(-1j * t * f, -1j * t * v, inplace=False)
        d.coeff = c.copy()
        ap = d.apply_diagonal_coulomb(f.astype(complex), vns.astype(complex),
                                      inplace=False)
        # through the public API: time_evolve with a DiagonalCoulomb
        wfn = fqe.Wavefunction([[na + nb, na - nb, norb]])
        wfn.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): c})
        te = wfn.time_evolve(t, fqe.get_diagonalcoulomb_hamiltonian(v))
        out.update({f"psi_{tag}": c, f"v_{tag}": v, f"vns_{tag}": vns,
                    f"f_{tag}": f, f"evolve_{tag}": numpy.asarray(ev),
                    f"apply_{tag}": numpy.asarray(ap),
                    f"time_evolve_{tag}": te.get_coeff((na + nb, na - nb))})
    save("diagonal_coulomb", **out)


def taylor_fixture():
    out = {}
    for norb, na, nb, t, acc, seed in [(6, 2, 2, 0.05, 1e-12, 0),
                                       (8, 4, 4, 0.05, 1e-12, 0),
                                       (5, 3, 1, 0.3, 1e-15, 1)]:
        h1, h2, rng = synthetic.integrals(norb, 2 * norb, seed)
        c = synthetic.wavefunction_coeff(math.comb(norb, na), math.comb(norb, nb), rng)
        wfn = fqe.Wavefunction([[na + nb, na - nb, norb]])
        wfn.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): c})
        ham = fqe.get_restricted_hamiltonian((h1, h2))
        res = wfn.apply_generated_unitary(t, "taylor", ham, accuracy=acc)
        tag = f"{norb}_{na}_{nb}"
        out.update({f"psi_{tag}": c, f"h1_{tag}": h1, f"h2_{tag}": h2,
                    f"t_{tag}": numpy.array(t), f"acc_{tag}": numpy.array(acc),
                    f"out_{tag}": res.get_coeff((na + nb, na - nb))})
    save("taylor", **out)


def dvec_fixture():
    out = {}
    for norb, na, nb, seed in [(4, 2, 1, 0), (5, 2, 2, 1)]:
        d = FqeData(na, nb, norb)
        rng = numpy.random.default_rng(4000 + seed)
        c = synthetic.wavefunction_coeff(d.lena(), d.lenb(), rng)
        d.coeff = c.copy()
        dv = d.calculate_dvec_spatial()
        co = d._calculate_coeff_spatial_with_dvec(dv)
        tag = f"{norb}_{na}_{nb}"
        out.update({f"psi_{tag}": c, f"dvec_{tag}": dv, f"coeff_{tag}": co})
    save("dvec", **out)


def davidson_fixture():
    """LiH (norb 6, 2+2 electrons) from the reference's own test data
    (tests/unittest_data/build_lih_data.py) with the reference Davidson's
    answer, and the norb-4 Hamiltonian h2[i,j,k,l] = 0.02 (i+k)(j+l) of
    fqe_data_test.py:763-771 with the reference Davidson's two lowest roots
    (its eigenvalue-change stopping rule leaves them ~4e-5 above the exact,
    four-fold degenerate -7.271991091302982 that the same test asserts)."""
    numpy.infty = numpy.inf  # removed in numpy 2; davidson.py:182 uses it
    sys.path.insert(0, os.path.join(ref_fqe.REF_ROOT, "tests"))
    from unittest_data.build_lih_data import build_lih_data
    from fqe.hamiltonians.restricted_hamiltonian import RestrictedHamiltonian
    from fqe.algorithm import davidson
    h1, h2, ground = build_lih_data("energy")
    ham = RestrictedHamiltonian((h1, h2))
    numpy.random.seed(3)
    w_lih, _ = davidson.davidson_diagonalization(ham, 2, 2, nroots=1)
    wfn = fqe.Wavefunction([[4, 0, 6]])
    wfn.set_wfn(strategy="from_data", raw_data={(4, 0): ground})
    e_lih = wfn.expectationValue(ham)
    norb = 4
    h2k = numpy.zeros((norb,) * 4, dtype=numpy.complex128)
    for i in range(norb):
        for j in range(norb):
            for k in range(norb):
                for l in range(norb):
                    h2k[i, j, k, l] += (i + k) * (j + l) * 0.02
    h1k = numpy.zeros((norb, norb), dtype=numpy.complex128)
    numpy.random.seed(4)
    w_k, _ = davidson.davidson_diagonalization(
        RestrictedHamiltonian((h1k, h2k)), 2, 2, nroots=2)
    save("davidson", lih_h1=numpy.asarray(h1), lih_h2=numpy.asarray(h2),
         lih_ground=numpy.asarray(ground),
         lih_e_test=numpy.array(-8.877719570384043),
         lih_e_expectation=numpy.array(e_lih),
         lih_e_ref_davidson=numpy.asarray(w_lih),
         k4_h1=h1k, k4_h2=h2k,
         k4_e_test=numpy.array(-7.271991091302982),
         k4_e_ref_davidson=numpy.asarray(w_k))


def rdm_fixture():
    """FqeData.rdm1 of the reference (fqe_data.py:1668-1724), both branches of
    its code-path switch, plus a transition RDM (bradata given)."""
    out = {}
    for norb, na, nb, seed in [(4, 2, 1, 0), (5, 2, 2, 1), (6, 3, 2, 2)]:
        rng = numpy.random.default_rng(5000 + seed)
        ket = FqeData(na, nb, norb)
        bra = FqeData(na, nb, norb)
        ket.coeff = synthetic.wavefunction_coeff(ket.lena(), ket.lenb(), rng)
        bra.coeff = synthetic.wavefunction_coeff(bra.lena(), bra.lenb(), rng)
        tag = f"{norb}_{na}_{nb}"
        fqe.settings.use_accelerated_code = True
        out[f"ket_{tag}"] = ket.coeff.copy()
        out[f"bra_{tag}"] = bra.coeff.copy()
        out[f"rdm1_{tag}"] = ket.rdm1()[0]
        out[f"trdm1_{tag}"] = ket.rdm1(bra)[0]
        fqe.settings.use_accelerated_code = False
        out[f"rdm1py_{tag}"] = ket.rdm1()[0]
        fqe.settings.use_accelerated_code = True
    save("rdm", **out)


def rdm12_fixture():
    """FqeData.rdm12 of the reference (fqe_data.py:1726-1760): the half-filling
    branch (blocked and plain numpy, :1762-1838) and the low-filling branch
    (C and python, :1840-2033), each with and without a bra (transition RDMs)."""
    out = {}
    for norb, na, nb, seed in [(4, 2, 1, 0), (5, 2, 2, 1), (6, 3, 2, 2),
                               (8, 2, 1, 3), (7, 1, 2, 4)]:
        rng = numpy.random.default_rng(6000 + seed)
        ket = FqeData(na, nb, norb)
        bra = FqeData(na, nb, norb)
        ket.coeff = synthetic.wavefunction_coeff(ket.lena(), ket.lenb(), rng)
        bra.coeff = synthetic.wavefunction_coeff(bra.lena(), bra.lenb(), rng)
        tag = f"{norb}_{na}_{nb}"
        out[f"ket_{tag}"] = ket.coeff.copy()
        out[f"bra_{tag}"] = bra.coeff.copy()
        # the filling threshold is fixed when an FqeData is made: objects
        # made with the accelerated switch on always take the half-filling
        # branch; objects made with it off take the low-filling branch below
        # 30 % filling (C or python by the switch at call time)
        for made, called, suffix in ((True, True, ""), (False, False, "py"),
                                     (False, True, "c")):
            fqe.settings.use_accelerated_code = made
            k2 = FqeData(na, nb, norb)
            b2 = FqeData(na, nb, norb)
            k2.coeff = ket.coeff.copy()
            b2.coeff = bra.coeff.copy()
            fqe.settings.use_accelerated_code = called
            r1, r2 = k2.rdm12()
            t1, t2 = k2.rdm12(b2)
            out[f"rdm1{suffix}_{tag}"] = r1
            out[f"rdm2{suffix}_{tag}"] = r2
            out[f"trdm1{suffix}_{tag}"] = t1
            out[f"trdm2{suffix}_{tag}"] = t2
        fqe.settings.use_accelerated_code = True
    save("rdm12", **out)


def spin_fixture():
    """FqeData.apply with spin-orbital operators (fqe_data.py:404-470 ->
    _apply_array_spin1 :533-608, _apply_array_spin12 :610-635): random
    complex h1 [2n, 2n] and h2 [2n]^4, alpha orbitals first."""
    out = {}
    for norb, na, nb, seed in [(4, 2, 2, 0), (5, 2, 1, 1), (5, 2, 3, 2),
                               (4, 0, 2, 3), (4, 3, 1, 4)]:
        rng = numpy.random.default_rng(7000 + seed)
        d = FqeData(na, nb, norb)
        d.coeff = synthetic.wavefunction_coeff(d.lena(), d.lenb(), rng)
        m = 2 * norb
        h1 = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
        h2 = rng.normal(size=(m,) * 4) + 1j * rng.normal(size=(m,) * 4)
        tag = f"{norb}_{na}_{nb}"
        out[f"psi_{tag}"] = d.coeff.copy()
        out[f"h1_{tag}"] = h1
        out[f"h2_{tag}"] = h2
        out[f"spin1_{tag}"] = d.apply((h1,)).coeff
        out[f"spin12_{tag}"] = d.apply((h1, h2)).coeff
    save("spin", **out)


def wfn_pickles_fixture():
    """The reference's own Wavefunction.apply golden data
    (tests/unittest_data/wavefunction/*.pickle, checked by
    tests/wavefunction_test.py:609-627): the restricted-Hamiltonian
    ('apply_array' with a RestrictedHamiltonian) and diagonal-Coulomb
    ('apply_dc') cases of the number-conserving wavefunctions, unpacked per
    sector into plain arrays."""
    import pickle
    from fqe.hamiltonians.restricted_hamiltonian import RestrictedHamiltonian
    src = os.path.join(ref_fqe.REF_ROOT, "tests", "unittest_data", "wavefunction")
    out = {}
    for f in sorted(os.listdir(src)):
        if not f.endswith(".pickle"):
            continue
        with open(os.path.join(src, f), "rb") as fh:
            data = pickle.load(fh)
        if not isinstance(data, dict) or "wfn" not in data:
            continue
        name = f[:-len(".pickle")].replace("-", "m")
        wfn = data["wfn"]
        if not wfn.conserve_number():
            # number-broken wavefunctions (the XX files) go through the
            # reference's beta-inversion (wavefunction.py:337-359): not on
            # this path
            continue
        norb = wfn.norb()
        cases = []
        arr = data.get("apply_array")
        if arr and isinstance(arr["hamil"], RestrictedHamiltonian) \
                and arr["wfn_out"] is not None:
            cases.append(("array", arr))
        dc = data.get("apply_dc")
        if dc and dc["wfn_out"] is not None:
            cases.append(("dc", dc))
        for kind, case in cases:
            ham = case["hamil"]
            tag = f"{name}_{kind}"
            out[f"norb_{tag}"] = numpy.array(norb)
            out[f"e0_{tag}"] = numpy.array(complex(ham.e_0()))
            if kind == "array":
                for r, t in enumerate(ham.tensors()):
                    out[f"t{r}_{tag}"] = numpy.asarray(t, dtype=numpy.complex128)
            else:
                out[f"diag_{tag}"] = numpy.asarray(ham._tensor[1], dtype=numpy.complex128)
                out[f"vij_{tag}"] = numpy.asarray(ham._tensor[2], dtype=numpy.complex128)
            for key in wfn.sectors():
                nele, sz = key
                na, nb = (nele + sz) // 2, (nele - sz) // 2
                sec = f"{tag}_{na}_{nb}"
                out[f"psi_{sec}"] = wfn.get_coeff(key).copy()
                out[f"out_{sec}"] = case["wfn_out"].get_coeff(key).copy()
    save("wfn_pickles", **out)


def transform_fixture():
    """Wavefunction.transform (wavefunction.py:813-959) with spatial (norb)
    and block-diagonal spin-orbital (2 norb) rotations, some close to a
    permutation so that the LU inside pivots; records the rotation, the
    returned permutation and the transformed sector."""
    from scipy.stats import unitary_group
    out = {}
    cases = [(4, 2, 1, 0, False, False), (5, 2, 2, 1, True, False),
             (6, 3, 2, 2, False, True), (5, 3, 1, 3, True, True),
             (4, 0, 2, 4, False, False)]
    for norb, na, nb, seed, near_perm, spin in cases:
        rng = numpy.random.default_rng(8000 + seed)

        def rot(k):
            u = unitary_group.rvs(norb, random_state=100 * seed + k)
            if near_perm:
                q = numpy.eye(norb)[rng.permutation(norb)]
                u, _ = numpy.linalg.qr(0.05 * u + q)
            return u
        if spin:
            U = numpy.zeros((2 * norb, 2 * norb), dtype=numpy.complex128)
            U[:norb, :norb] = rot(0)
            U[norb:, norb:] = rot(1)
        else:
            U = rot(0)
        w = fqe.Wavefunction([[na + nb, na - nb, norb]])
        lena, lenb = math.comb(norb, na), math.comb(norb, nb)
        psi = synthetic.wavefunction_coeff(lena, lenb, rng)
        w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi.copy()})
        perm, _, _, res = w.transform(U)
        tag = f"{norb}_{na}_{nb}_{seed}"
        out[f"psi_{tag}"] = psi
        out[f"rot_{tag}"] = U
        out[f"perm_{tag}"] = perm
        out[f"out_{tag}"] = res.get_coeff((na + nb, na - nb)).copy()
    save("transform", **out)


def chebyshev_fixture():
    """Wavefunction.apply_generated_unitary(time, 'chebyshev', ...)
    (wavefunction.py:570-606) for restricted Hamiltonians with and without
    e_0, spectral limits from the dense spectrum widened by 5 %."""
    from fqe.hamiltonians.restricted_hamiltonian import RestrictedHamiltonian
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    out = {}
    for norb, na, nb, seed, e0, t in [(4, 2, 1, 0, 0.0, 0.3), (5, 2, 2, 1, 0.7 - 0.2j, 0.25),
                                       (6, 3, 2, 2, 0.0, 0.1)]:
        h1, h2, psi = synthetic.sector(norb, na, nb, 2 * norb, seed)
        g = oracle.graph(norb, na, nb)
        H = oracle.dense_hamiltonian(h1, h2, g)
        w = numpy.linalg.eigvalsh(0.5 * (H + H.conj().T))
        pad = 0.05 * (w[-1] - w[0])
        lim = [float(w[0] - pad), float(w[-1] + pad)]
        ham = RestrictedHamiltonian((h1, h2), e_0=e0)
        wfn = fqe.Wavefunction([[na + nb, na - nb, norb]])
        wfn.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi.copy()})
        res = wfn.apply_generated_unitary(t, "chebyshev", ham, accuracy=1e-13,
                                          expansion=200, spec_lim=lim)
        tag = f"{norb}_{na}_{nb}"
        out[f"psi_{tag}"] = psi
        out[f"h1_{tag}"] = h1
        out[f"h2_{tag}"] = h2
        out[f"e0_{tag}"] = numpy.array(complex(e0))
        out[f"t_{tag}"] = numpy.array(t)
        out[f"lim_{tag}"] = numpy.array(lim)
        out[f"out_{tag}"] = res.get_coeff((na + nb, na - nb)).copy()
    save("chebyshev", **out)


def quadratic_fixture():
    """Wavefunction.time_evolve with a quadratic (one-body) restricted
    Hamiltonian (wavefunction.py:1008-1032: diagonalising transformation,
    transform, diagonal evolution, transform back), with e_0."""
    out = {}
    for norb, na, nb, seed in [(4, 2, 1, 0), (5, 2, 2, 1), (6, 3, 2, 2), (6, 3, 3, 3)]:
        rng = numpy.random.default_rng(9100 + seed)
        a = rng.normal(size=(norb, norb)) + 1j * rng.normal(size=(norb, norb))
        h1 = 0.5 * (a + a.conj().T)
        e0 = 0.3 - 0.1 * seed
        lena, lenb = math.comb(norb, na), math.comb(norb, nb)
        psi = synthetic.wavefunction_coeff(lena, lenb, rng)
        w = fqe.Wavefunction([[na + nb, na - nb, norb]])
        w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi.copy()})
        ham = fqe.get_restricted_hamiltonian((h1,), e_0=e0)
        t = 0.7 + 0.1 * seed
        res = w.time_evolve(t, ham)
        tag = f"{norb}_{na}_{nb}_{seed}"
        out[f"psi_{tag}"] = psi
        out[f"h1_{tag}"] = h1
        out[f"e0_{tag}"] = numpy.array(e0)
        out[f"t_{tag}"] = numpy.array(t)
        out[f"out_{tag}"] = res.get_coeff((na + nb, na - nb)).copy()
    save("quadratic", **out)


def saved_wfn_fixture():
    """A file written by the reference's own Wavefunction.save
    (wavefunction.py:747-765: a pickled list [symmetry map, conserved,
    conserve_spin, conserve_number, norb, [key, FqeData], ...]) for three
    sectors of norb 4, with the coefficients beside it in saved_wfn.npz."""
    rng = numpy.random.default_rng(21)
    wfn = fqe.Wavefunction([[4, 0, 4], [4, 2, 4], [4, -2, 4]])
    out = {}
    for key in wfn.sectors():
        shape = wfn.get_coeff(key).shape
        c = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        wfn.set_wfn(strategy="from_data", raw_data={key: c})
        out[f"coeff_{key[0]}_{key[1]}"] = c
    wfn.save("ref_saved_wfn.pickle", path=HERE)
    print("wrote", os.path.join(HERE, "ref_saved_wfn.pickle"))
    save("saved_wfn", **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["graph", "apply", "dc", "taylor", "dvec",
                             "davidson", "rdm", "rdm12", "spin", "wfn_pickles",
                             "transform", "chebyshev", "graph_pickles", "saved_wfn",
                             "quadratic"]
    for name in which:
        globals()[name + "_fixture"]()
