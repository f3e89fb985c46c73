"""The spin-orbital (generalised) one- and two-body apply on the GPU
(fqegpu_ham_create_spin), against the reference's own outputs
(tests/golden/spin.npz: FqeData.apply with 2n-dimensional operators, i.e.
_apply_array_spin1 fqe_data.py:533-563 and _apply_array_spin12_lm
:743-773) and against the oracle's restatement on seeded unrestricted
integrals, FP64 (<= 1e-12) and tensor cores (<= 1e-10)."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(numpy.linalg.norm(a - b) / numpy.linalg.norm(b))


def _apply(gpu, norb, na, nb, psi, tensors, precision="fp64"):
    from fqe_gb300 import settings
    w = gpu.Wavefunction([[na + nb, na - nb, norb]])
    w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi})
    old = settings.precision
    settings.precision = precision
    try:
        return w.apply(tensors).get_coeff((na + nb, na - nb)).cpu().numpy()
    finally:
        settings.precision = old


def test_spin_apply_matches_reference_outputs(gpu, golden):
    gd = golden("spin")
    for key in [k for k in gd if k.startswith("spin12_")]:
        tag = key[7:]
        norb, na, nb = map(int, tag.split("_"))
        psi, h1, h2 = gd["psi_" + tag], gd["h1_" + tag], gd["h2_" + tag]
        out1 = _apply(gpu, norb, na, nb, psi, (h1,))
        assert numpy.abs(out1 - gd["spin1_" + tag]).max() < 1e-12
        out12 = _apply(gpu, norb, na, nb, psi, (h1, h2))
        scale = max(1.0, numpy.abs(gd[key]).max())
        assert numpy.abs(out12 - gd[key]).max() < 1e-12 * scale


def _unrestricted(norb, seed):
    """Real unrestricted integrals in spin orbitals: separate alpha and beta
    one-body blocks and Cholesky factors (chemist (ij|kl) per spin pair),
    mapped to FQE's h2[I,J,K,L] (a+_I a+_J a_K a_L) as -1/2 (IK|JL)."""
    from fqe_gb300 import synthetic
    h1a, _, rng = synthetic.integrals(norb, 2 * norb, seed)
    h1b, _, _ = synthetic.integrals(norb, 2 * norb, seed + 100)
    La = rng.normal(0.0, 0.3, size=(2 * norb, norb, norb))
    La = 0.5 * (La + La.transpose(0, 2, 1))
    Lb = La + rng.normal(0.0, 0.05, size=La.shape)
    Lb = 0.5 * (Lb + Lb.transpose(0, 2, 1))
    m = 2 * norb
    H1 = numpy.zeros((m, m))
    H1[:norb, :norb] = h1a
    H1[norb:, norb:] = h1b
    eri = numpy.zeros((m,) * 4)
    L = {0: La, 1: Lb}
    for s in (0, 1):
        for t in (0, 1):
            blk = numpy.einsum('xij,xkl->ijkl', L[s], L[t])
            eri[s * norb:(s + 1) * norb, s * norb:(s + 1) * norb,
                t * norb:(t + 1) * norb, t * norb:(t + 1) * norb] = blk
    H2 = -0.5 * numpy.einsum('ikjl->ijkl', eri)
    return H1, numpy.ascontiguousarray(H2)


@pytest.mark.parametrize("norb,na,nb", [(6, 3, 2), (8, 4, 4), (9, 5, 3), (10, 5, 5)])
@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_spin_apply_unrestricted_integrals(gpu, oracle, norb, na, nb, precision):
    from fqe_gb300 import synthetic
    H1, H2 = _unrestricted(norb, norb + na)
    _, _, psi = synthetic.sector(norb, na, nb, 2 * norb, seed=norb)
    g = oracle.graph(norb, na, nb)
    want = oracle.apply_spin12(psi, H1, H2, g)
    got = _apply(gpu, norb, na, nb, psi, (H1, H2), precision)
    tol = 1e-12 if precision == "fp64" else 1e-10
    assert _rel(got, want) < tol
    # one-body only
    want1 = oracle.apply_spin1(psi, H1, g)
    got1 = _apply(gpu, norb, na, nb, psi, (H1,), precision)
    assert _rel(got1, want1) < tol


def test_spin_free_operator_equals_restricted_apply(gpu):
    from fqe_gb300 import synthetic
    norb, na, nb = 8, 4, 3
    h1, h2, psi = synthetic.sector(norb, na, nb, 16, seed=2)
    m = 2 * norb
    H1 = numpy.kron(numpy.eye(2), h1)
    H2 = numpy.zeros((m,) * 4)
    for s in (slice(0, norb), slice(norb, m)):
        for t in (slice(0, norb), slice(norb, m)):
            H2[s, t, s, t] = h2
    a = _apply(gpu, norb, na, nb, psi, (h1, h2))
    b = _apply(gpu, norb, na, nb, psi, (H1, H2))
    assert _rel(b, a) < 1e-12


def test_spin_taylor_matches_oracle(gpu, oracle):
    from fqe_gb300 import settings, synthetic
    norb, na, nb = 8, 4, 3
    H1, H2 = _unrestricted(norb, 5)
    _, _, psi = synthetic.sector(norb, na, nb, 16, seed=5)
    g = oracle.graph(norb, na, nb)
    # the reference's Taylor loop with the spin-orbital apply as H
    work = psi.copy()
    ref = psi.copy()
    import math
    for k in range(1, 80):
        work = oracle.apply_spin12(work, -0.05j * H1, -0.05j * H2, g)
        ref += work / math.factorial(k)
        if numpy.linalg.norm(work) / math.factorial(k) < 1e-12:
            break
    w = gpu.Wavefunction([[na + nb, na - nb, norb]])
    w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi})
    ham = gpu.General((H1, H2))
    for prec, tol in (("fp64", 1e-12), ("ozaki", 1e-10)):
        old = settings.precision
        settings.precision = prec
        try:
            ev = w.apply_generated_unitary(0.05, "taylor", ham, accuracy=1e-12,
                                           expansion=80)
        finally:
            settings.precision = old
        assert _rel(ev.get_coeff((na + nb, na - nb)).cpu().numpy(), ref) < tol
