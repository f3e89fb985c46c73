"""The benchmark's other configurations as parity cases (sizes the oracle
finishes in seconds, plus size-independent properties at full size):

* uneven sectors over norb {8, 10, 12}, each with its own seeded integrals
  (seed = index), one apply and a Taylor evolution t = 0.1 to 1e-10, FP64 and
  tensor-core paths against the oracle;
* norb 16: a (3, 3) sector (P = 136 compressed pairs: the tensor-core form
  runs two passes of output pairs) against the oracle, a short Taylor
  evolution, and the full (8, 8) sector through Hermiticity of the apply.
"""

import math

import numpy
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_OZ = 1e-10

UNEVEN = [(8, 5, 3), (8, 4, 4), (8, 3, 5), (10, 5, 5), (10, 6, 4),
          (10, 4, 5), (12, 6, 6), (12, 5, 6)]


def _rel(a, b):
    return numpy.linalg.norm(a - b) / max(numpy.linalg.norm(b), 1e-300)


def _wfn(gpu, norb, na, nb, coeff):
    w = gpu.Wavefunction([[na + nb, na - nb, norb]])
    w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): coeff})
    return w


@pytest.mark.parametrize("index", range(len(UNEVEN)))
@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_uneven_sector_apply_and_taylor(gpu, oracle, index, precision):
    from fqe_gb300 import settings, synthetic
    norb, na, nb = UNEVEN[index]
    h1, h2, psi = synthetic.sector(norb, na, nb, 2 * norb, seed=index)
    g = oracle.graph(norb, na, nb)
    ham = gpu.RestrictedHamiltonian((h1, h2))
    tol = TOL_FP64 if precision == "fp64" else TOL_OZ
    old = settings.precision
    settings.precision = precision
    try:
        w = _wfn(gpu, norb, na, nb, psi)
        out = w.apply(ham).get_coeff((na + nb, na - nb)).cpu().numpy()
        want = oracle.apply_restricted(psi, (h1, h2), 0.0, g)
        assert _rel(out, want) < tol
        # ||0.1 H|| reaches ~7 at norb 12 with these integrals: the series
        # needs more than the default 30 terms
        ev = w.apply_generated_unitary(0.1, "taylor", ham, accuracy=1e-10,
                                       expansion=80)
        got = ev.get_coeff((na + nb, na - nb)).cpu().numpy()
        ref, _ = oracle.taylor_evolve(psi, (h1, h2), 0.0, 0.1, g, accuracy=1e-10,
                                      expansion=80)
        assert _rel(got, ref) < tol
        assert abs(numpy.linalg.norm(got) - 1.0) < 1e-9  # unitary to 1e-10 steps
    finally:
        settings.precision = old


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_norb16_sector(gpu, oracle, precision):
    from fqe_gb300 import settings, synthetic
    norb, na, nb = 16, 3, 3
    h1, h2, psi = synthetic.sector(norb, na, nb, 32, seed=0)
    g = oracle.graph(norb, na, nb)
    ham = gpu.RestrictedHamiltonian((h1, h2))
    old = settings.precision
    settings.precision = precision
    try:
        w = _wfn(gpu, norb, na, nb, psi)
        out = w.apply(ham).get_coeff((na + nb, na - nb)).cpu().numpy()
        want = oracle.apply_restricted(psi, (h1, h2), 0.0, g)
        # P = 136: the tensor-core form runs in two passes of 80 output pairs
        tol = TOL_FP64 if precision == "fp64" else TOL_OZ
        assert _rel(out, want) < tol
        # two Taylor steps of dt = 0.05: norm and fidelity against the oracle
        cur, ref = w, psi
        for _ in range(2):
            cur = cur.apply_generated_unitary(0.05, "taylor", ham, accuracy=1e-12)
            ref, _ = oracle.taylor_evolve(ref, (h1, h2), 0.0, 0.05, g,
                                          accuracy=1e-12)
            got = cur.get_coeff((na + nb, na - nb)).cpu().numpy()
            assert abs(numpy.linalg.norm(got) - 1.0) < 10 * tol
            assert abs(abs(numpy.vdot(ref.ravel(), got.ravel())) - 1.0) < 10 * tol
    finally:
        settings.precision = old


def test_norb16_full_sector_hermitian(gpu):
    # (8, 8): 165,636,900 determinants, streamed in beta-column blocks;
    # <phi|H psi> = conj(<psi|H phi>) for two random states
    import torch
    from fqe_gb300 import synthetic
    from fqe_gb300.fqe_data import FqeData
    norb = 16
    h1, h2, rng = synthetic.integrals(norb, 32, seed=0)
    n = math.comb(16, 8)
    ham = (h1, h2)
    vecs = []
    for s in range(2):
        g = torch.Generator(device="cuda").manual_seed(100 + s)
        c = torch.complex(torch.randn(n, n, generator=g, device="cuda",
                                      dtype=torch.float64),
                          torch.randn(n, n, generator=g, device="cuda",
                                      dtype=torch.float64))
        c /= torch.linalg.vector_norm(c)
        d = FqeData(8, 8, norb)
        d.coeff.copy_(c)
        vecs.append(d)
        del c
    hx = vecs[0].apply(ham)
    a = complex(torch.vdot(vecs[1].coeff.reshape(-1), hx.coeff.reshape(-1)))
    del hx
    hy = vecs[1].apply(ham)
    b = complex(torch.vdot(vecs[0].coeff.reshape(-1), hy.coeff.reshape(-1)))
    assert abs(a - b.conjugate()) <= 1e-12 * max(abs(a), 1e-300) + 1e-14
    assert math.isfinite(abs(a))
