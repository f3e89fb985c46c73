"""Davidson (A12) on the GPU against the oracle's dense spectrum and the
reference's known answers (tests/golden/davidson.npz, from
tests/golden/make_golden.py)."""

import numpy
import pytest

pytestmark = pytest.mark.gpu

E_TOL = 1e-9  # converged eigenvalue vs exact (residual tolerance 1e-6)


def _dense_low(oracle, h1, h2, norb, na, nb, k):
    g = oracle.graph(norb, na, nb)
    H = oracle.dense_hamiltonian(h1.astype(complex), h2.astype(complex), g)
    return numpy.linalg.eigvalsh(0.5 * (H + H.conj().T))[:k]


def test_lih_ground_state(gpu, golden):
    # tests/davidson_test.py:26-113 of the reference: LiH (norb 6, 2+2),
    # eref = -8.877719570384043, both entry points.
    from fqe_gb300 import davidson
    gd = golden("davidson")
    ham = gpu.RestrictedHamiltonian((gd["lih_h1"], gd["lih_h2"]))
    w, v = davidson.davidson_diagonalization(ham, 2, 2)
    assert abs(w[0] - float(gd["lih_e_test"])) < E_TOL
    assert abs(v[0].expectationValue(ham) - w[0]) < E_TOL
    ground = gd["lih_ground"]
    x = v[0].get_coeff((4, 0)).cpu().numpy()
    assert abs(abs(numpy.vdot(ground.ravel(), x.ravel())) - 1.0) < 1e-8
    # davidsonliu_fqe with the reference test's two HF-like guesses
    guesses = []
    for idx in (0, 2):  # strings 0b000011 and 0b000110 in both spins
        c = numpy.zeros((15, 15), dtype=complex)
        c[idx, idx] = 1.0
        wf = gpu.Wavefunction([[4, 0, 6]])
        wf.set_wfn(strategy="from_data", raw_data={(4, 0): c})
        guesses.append(wf)
    w2, _ = davidson.davidsonliu_fqe(ham, 1, guesses, nele=4, sz=0, norb=6)
    assert abs(w2[0] - float(gd["lih_e_test"])) < E_TOL


def test_degenerate_known_answer(gpu, golden):
    # fqe_data_test.py:763-771: h2[i,j,k,l] = 0.02 (i+k)(j+l), norb 4, 2+2;
    # -7.271991091302982 is four-fold degenerate.  The reference Davidson
    # stops ~4e-5 above it; the residual rule reaches it.
    from fqe_gb300 import davidson
    gd = golden("davidson")
    ham = gpu.RestrictedHamiltonian((gd["k4_h1"], gd["k4_h2"]))
    res = davidson.davidson(ham, 2, 2, nroots=4)
    assert res.converged
    numpy.testing.assert_allclose(res.eigenvalues, float(gd["k4_e_test"]),
                                  atol=E_TOL, rtol=0)
    assert res.eigenvalues[0] < gd["k4_e_ref_davidson"][0] - 1e-6


@pytest.mark.parametrize("norb,na,nb,nroots,seed", [
    (6, 3, 3, 3, 11), (7, 3, 2, 2, 12), (7, 3, 3, 1, 13)])
def test_synthetic_vs_dense(gpu, oracle, norb, na, nb, nroots, seed):
    from fqe_gb300 import davidson, synthetic
    h1, h2, _ = synthetic.integrals(norb, 2 * norb, seed)
    ham = gpu.RestrictedHamiltonian((h1, h2), e_0=0.25)
    res = davidson.davidson(ham, na, nb, nroots=nroots, block=nroots + 1)
    assert res.converged
    exact = _dense_low(oracle, h1, h2, norb, na, nb, nroots) + 0.25
    numpy.testing.assert_allclose(res.eigenvalues, exact, atol=E_TOL, rtol=0)


def test_ozaki_precision_same_energy(gpu, oracle):
    # the tensor-core H·psi (relative error <= 1e-10 per apply) converges to
    # the same root as the FP64 path
    from fqe_gb300 import davidson, synthetic
    h1, h2, _ = synthetic.integrals(8, 16, 21)
    ham = gpu.RestrictedHamiltonian((h1, h2))
    r64 = davidson.davidson(ham, 4, 4, precision="fp64")
    roz = davidson.davidson(ham, 4, 4, precision="ozaki")
    assert r64.converged and roz.converged
    assert abs(r64.eigenvalues[0] - roz.eigenvalues[0]) < E_TOL


def test_preconditioner_kernel(gpu):
    import torch
    from fqe_gb300 import _lib
    from fqe_gb300.fqe_data import _ptr, _stream
    rng = numpy.random.default_rng(5)
    n = 100003
    r = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    d = rng.standard_normal(n)
    d[:7] = 0.3  # |theta - d| below the floor
    theta, floor_ = 0.3 + 1e-9, 1e-4
    rt = torch.from_numpy(r).cuda()
    dt = torch.from_numpy(d).cuda()
    tt = torch.empty_like(rt)
    _lib.call("fqegpu_precondition", n, _ptr(rt), _ptr(dt), theta, floor_,
              _ptr(tt), _stream())
    den = theta - d
    small = numpy.abs(den) < floor_
    den[small] = numpy.where(den[small] < 0, -floor_, floor_)
    want = r.real / den + 1j * (r.imag / den)
    # the kernel multiplies by 1/den: at most one extra rounding
    numpy.testing.assert_allclose(tt.cpu().numpy(), want, rtol=4e-16, atol=0)
    with pytest.raises(ValueError):
        _lib.call("fqegpu_precondition", n, _ptr(rt), _ptr(dt), theta, 0.0,
                  _ptr(tt), _stream())


def test_errors(gpu, golden):
    from fqe_gb300 import davidson
    gd = golden("davidson")
    ham = gpu.RestrictedHamiltonian((gd["lih_h1"], gd["lih_h2"]))
    with pytest.raises(ValueError):
        davidson.davidsonliu_fqe(ham, 0, [gpu.Wavefunction([[4, 0, 6]])],
                                 nele=4, sz=0, norb=6)
    a = gpu.Wavefunction([[4, 0, 6]])
    b = gpu.Wavefunction([[4, 2, 6]])
    with pytest.raises(TypeError):
        davidson.davidsonliu_fqe(ham, 1, [a, b], nele=4, sz=0, norb=6)
    with pytest.raises(ValueError):
        davidson.davidson(ham, 2, 2, nroots=226)


def test_block_vector_ops(gpu):
    # fqegpu_block_vdot / fqegpu_block_axpy against numpy, k up to 70
    # (two chunks of at most 64 on the host side)
    import torch
    from fqe_gb300 import davidson
    rng = numpy.random.default_rng(9)
    n = 20011
    for k in (1, 7, 64, 70):
        vs_h = [rng.normal(size=n) + 1j * rng.normal(size=n) for _ in range(k)]
        t_h = rng.normal(size=n) + 1j * rng.normal(size=n)
        vs = [torch.from_numpy(v).cuda() for v in vs_h]
        t = torch.from_numpy(t_h).cuda()
        got = davidson._block_vdot(vs, t)
        want = numpy.array([numpy.vdot(v, t_h) for v in vs_h])
        numpy.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-10)
        coef = rng.normal(size=k) + 1j * rng.normal(size=k)
        davidson._block_axpy(coef, vs, t)
        want_t = t_h + sum(c * v for c, v in zip(coef, vs_h))
        numpy.testing.assert_allclose(t.cpu().numpy(), want_t, rtol=1e-13,
                                      atol=1e-12)
        # deterministic: the same reduction twice gives identical bits
        assert numpy.array_equal(davidson._block_vdot(vs, t),
                                 davidson._block_vdot(vs, t))
