"""Tensor-core (tcgen05, Ozaki-split BF16) contraction: parity with the FP64
path and the oracle.  Tolerance: relative 2-norm error <= 1e-10 (the stated
target for the split form)."""

import numpy
import pytest

pytestmark = pytest.mark.gpu

TOL_OZ = 1e-10


def _rel(a, b):
    return numpy.linalg.norm(a - b) / max(numpy.linalg.norm(b), 1e-300)


@pytest.fixture
def ozaki(gpu):
    from fqe_gb300 import settings
    settings.precision = "ozaki"
    yield gpu
    settings.precision = "fp64"


def _apply(gpu, norb, na, nb, h1, h2, psi):
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data", raw_data=psi)
    return d.apply((h1, h2)).to_numpy()


@pytest.mark.parametrize("norb,na,nb", [(4, 2, 2), (6, 3, 2), (8, 4, 4), (9, 4, 3),
                                        (10, 5, 5), (11, 3, 6), (12, 6, 6), (13, 6, 5),
                                        # an empty or full spin: one alpha or beta string
                                        (9, 0, 4), (8, 8, 2), (7, 3, 0)])
def test_ozaki_matches_fp64_and_oracle(ozaki, oracle, norb, na, nb):
    from fqe_gb300 import synthetic, settings
    h1, h2, rng = synthetic.integrals(norb, norb + 4, 100 + norb)
    g = oracle.graph(norb, na, nb)
    psi = synthetic.wavefunction_coeff(g.lena, g.lenb, rng)
    out = _apply(ozaki, norb, na, nb, h1, h2, psi)
    settings.precision = "fp64"
    ref64 = _apply(ozaki, norb, na, nb, h1, h2, psi)
    settings.precision = "ozaki"
    assert _rel(out, ref64) < TOL_OZ
    if norb <= 10:
        assert _rel(out, oracle.apply_spatial12(psi, h1, h2, g)) < TOL_OZ


def test_ozaki_peaked_wavefunction(ozaki, oracle):
    from fqe_gb300 import synthetic
    norb, na, nb = 10, 5, 5
    h1, h2, rng = synthetic.integrals(norb, 12, 5)
    g = oracle.graph(norb, na, nb)
    psi = 1e-6 * (rng.normal(size=(g.lena, g.lenb)) + 1j * rng.normal(size=(g.lena, g.lenb)))
    psi[0, 0] = 0.99
    psi[17, 3] = -0.1j
    out = _apply(ozaki, norb, na, nb, h1, h2, psi)
    assert _rel(out, oracle.apply_spatial12(psi, h1, h2, g)) < TOL_OZ


def test_ozaki_imaginary_scale_and_e0(ozaki, oracle):
    """-i t H (the Taylor operator) and e_0 ride through the same kernel."""
    from fqe_gb300 import synthetic
    norb, na, nb = 8, 4, 3
    h1, h2, rng = synthetic.integrals(norb, 10, 9)
    g = oracle.graph(norb, na, nb)
    psi = synthetic.wavefunction_coeff(g.lena, g.lenb, rng)
    out = _apply(ozaki, norb, na, nb, -0.05j * h1, -0.05j * h2, psi)
    assert _rel(out, oracle.apply_spatial12(psi, -0.05j * h1, -0.05j * h2, g)) < TOL_OZ
    wfn = ozaki.Wavefunction([[na + nb, na - nb, norb]])
    wfn.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi})
    res = wfn.apply(ozaki.get_restricted_hamiltonian((h1, h2), e_0=2.5))
    ref = oracle.apply_restricted(psi, (h1, h2), 2.5, g)
    assert _rel(res.get_coeff((na + nb, na - nb)).cpu().numpy(), ref) < TOL_OZ


def test_ozaki_taylor(ozaki, oracle, golden):
    gd = golden("taylor")
    for key in [k for k in gd if k.startswith("out_")]:
        tag = key[4:]
        norb, na, nb = map(int, tag.split("_"))
        wfn = ozaki.Wavefunction([[na + nb, na - nb, norb]])
        wfn.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): gd["psi_" + tag]})
        ham = ozaki.get_restricted_hamiltonian((gd["h1_" + tag], gd["h2_" + tag]))
        out = wfn.apply_generated_unitary(float(gd["t_" + tag]), "taylor", ham,
                                          accuracy=float(gd["acc_" + tag]))
        assert _rel(out.get_coeff((na + nb, na - nb)).cpu().numpy(), gd[key]) < TOL_OZ


def test_ozaki_complex_integrals_run_fp64_kernel(ozaki, oracle):
    rng = numpy.random.default_rng(8)
    norb, na, nb = 6, 3, 2
    h1 = rng.normal(size=(norb,) * 2) + 1j * rng.normal(size=(norb,) * 2)
    h2 = rng.normal(size=(norb,) * 4) + 1j * rng.normal(size=(norb,) * 4)
    g = oracle.graph(norb, na, nb)
    psi = rng.normal(size=(g.lena, g.lenb)) + 1j * rng.normal(size=(g.lena, g.lenb))
    out = _apply(ozaki, norb, na, nb, h1, h2, psi)
    assert _rel(out, oracle.apply_spatial12(psi, h1, h2, g)) < 1e-12


def test_ozaki_deterministic(ozaki):
    from fqe_gb300 import synthetic
    h1, h2, rng = synthetic.integrals(10, 12, 3)
    psi = synthetic.wavefunction_coeff(252, 210, rng)
    a = _apply(ozaki, 10, 5, 4, h1, h2, psi)
    b = _apply(ozaki, 10, 5, 4, h1, h2, psi)
    assert numpy.array_equal(a, b)


def test_plans_of_different_sizes_coexist(gpu, ozaki):
    # a large sector's plan first, then a small one, then the large one again:
    # the contraction kernel's shared-memory limit must fit every plan
    from fqe_gb300 import synthetic
    outs = []
    # shared memory per plan: norb 12 ~224 KB, norb 8 ~215 KB
    for norb, na, nb in [(12, 6, 6), (8, 4, 4), (12, 6, 6)]:
        h1, h2, psi = synthetic.sector(norb, na, nb, 2 * norb, seed=norb)
        d = gpu.FqeData(na, nb, norb)
        d.set_wfn(strategy="from_data", raw_data=psi)
        outs.append(d.apply((h1, h2)).coeff.cpu().numpy())
    assert numpy.array_equal(outs[0], outs[2])


@pytest.mark.parametrize("norb,na,nb,limit", [
    (10, 5, 5, 40 << 20),     # beta-column blocks of 64 columns
    (10, 5, 4, 7 << 20),      # blocks of 32 columns (the narrowest)
    (17, 2, 2, None),         # P = 153: two passes of output pairs
    (17, 3, 2, 40 << 20)])    # both at once
def test_blocks_and_passes(gpu, oracle, ozaki, norb, na, nb, limit):
    from fqe_gb300 import _lib, synthetic
    from fqe_gb300.fqe_data import ham_for
    h1, h2, psi = synthetic.sector(norb, na, nb, 2 * norb, seed=norb + na)
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data", raw_data=psi)
    ham = ham_for(d._core, h1, h2)
    if limit is not None:
        _lib.call("fqegpu_ham_set_scratch_limit", ham.handle, limit)
    out = d._run_apply(ham, alpha=0.5, beta=-0.25).cpu().numpy()
    g = oracle.graph(norb, na, nb)
    want = 0.5 * oracle.apply_spatial12(psi, h1, h2, g) - 0.25 * psi
    err = numpy.linalg.norm(out - want) / numpy.linalg.norm(want)
    assert err < TOL_OZ, err
