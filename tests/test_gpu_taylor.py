"""The device-resident Taylor series (fqegpu_taylor: one CUDA graph with a
conditional loop) and many sectors' series in one graph
(fqegpu_batch_taylor_*), against the oracle's restatement of
Wavefunction.apply_generated_unitary 'taylor' (wavefunction.py:553-568) and
against each other; the Chebyshev propagator (wavefunction.py:570-606) on the
GPU against the reference's own outputs."""

import numpy
import pytest

pytestmark = pytest.mark.gpu

SECTORS = [(8, 5, 3), (8, 4, 4), (10, 5, 5), (10, 6, 4), (12, 6, 6), (9, 4, 5),
           (8, 3, 5), (10, 4, 5), (12, 5, 6), (8, 2, 3)]


def _rel(a, b):
    return float(numpy.linalg.norm(a - b) / numpy.linalg.norm(b))


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_taylor_graph_reuse_and_terms(gpu, oracle, precision):
    from fqe_gb300 import settings, synthetic
    norb, na, nb = 10, 5, 5
    h1, h2, psi = synthetic.sector(norb, na, nb, 20, seed=1)
    ham = gpu.RestrictedHamiltonian((h1, h2), e_0=-0.3)
    g = oracle.graph(norb, na, nb)
    ref, terms = oracle.taylor_evolve(psi, (h1, h2), -0.3, 0.1, g, accuracy=1e-11,
                                      expansion=80)
    old = settings.precision
    settings.precision = precision
    try:
        w = gpu.Wavefunction([[na + nb, na - nb, norb]])
        w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi})
        outs = []
        for _ in range(3):  # the second and third calls reuse the graph
            ev = w.apply_generated_unitary(0.1, "taylor", ham, accuracy=1e-11,
                                           expansion=80)
            outs.append(ev.get_coeff((na + nb, na - nb)).cpu().numpy())
            assert ev._taylor_terms == terms
        assert numpy.array_equal(outs[0], outs[1])
        assert numpy.array_equal(outs[0], outs[2])
        tol = 1e-12 if precision == "fp64" else 1e-10
        assert _rel(outs[0], ref) < tol
        with pytest.raises(RuntimeError, match="expansion limit"):
            w.apply_generated_unitary(0.1, "taylor", ham, accuracy=1e-11, expansion=4)
    finally:
        settings.precision = old


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_batch_taylor_matches_single_series(gpu, oracle, precision):
    import torch
    from fqe_gb300 import settings, synthetic
    from fqe_gb300.batch import BatchTaylor
    datas, arrays, psis = [], [], []
    for i, (norb, na, nb) in enumerate(SECTORS):
        h1, h2, psi = synthetic.sector(norb, na, nb, 2 * norb, seed=i)
        d = gpu.FqeData(na, nb, norb)
        d.set_wfn(strategy="from_data", raw_data=psi)
        datas.append(d)
        arrays.append((h1, h2))
        psis.append(psi)
    bt = BatchTaylor(datas, arrays, 0.1, accuracy=1e-10, expansion=80,
                     precision=precision)
    bt.launch()
    terms = bt.terms()
    got = [d.coeff.cpu().numpy() for d in datas]
    old = settings.precision
    settings.precision = precision
    try:
        for i, (norb, na, nb) in enumerate(SECTORS):
            w = gpu.Wavefunction([[na + nb, na - nb, norb]])
            w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psis[i]})
            ham = gpu.RestrictedHamiltonian(arrays[i])
            ev = w.apply_generated_unitary(0.1, "taylor", ham, accuracy=1e-10,
                                           expansion=80)
            assert ev._taylor_terms == terms[i]
            assert numpy.array_equal(ev.get_coeff((na + nb, na - nb)).cpu().numpy(),
                                     got[i])
    finally:
        settings.precision = old
    tol = 1e-12 if precision == "fp64" else 1e-10
    for i in (0, 4, 9):
        norb, na, nb = SECTORS[i]
        ref, nt = oracle.taylor_evolve(psis[i], arrays[i], 0.0, 0.1,
                                       oracle.graph(norb, na, nb), accuracy=1e-10,
                                       expansion=80)
        assert nt == terms[i]
        assert _rel(got[i], ref) < tol
    # a second launch evolves every sector once more, in place
    bt.launch()
    bt.terms()
    torch.cuda.synchronize()
    for i in (0, 4):
        norb, na, nb = SECTORS[i]
        ref, _ = oracle.taylor_evolve(psis[i], arrays[i], 0.0, 0.2,
                                      oracle.graph(norb, na, nb), accuracy=1e-10,
                                      expansion=120)
        assert _rel(datas[i].coeff.cpu().numpy(), ref) < 100 * tol


def test_chebyshev_on_gpu_matches_reference(gpu, golden):
    gd = golden("chebyshev")
    for key in [k for k in gd if k.startswith("out_")]:
        tag = key[4:]
        norb, na, nb = map(int, tag.split("_"))
        ham = gpu.RestrictedHamiltonian((gd["h1_" + tag], gd["h2_" + tag]),
                                        e_0=complex(gd["e0_" + tag]))
        w = gpu.Wavefunction([[na + nb, na - nb, norb]])
        w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): gd["psi_" + tag]})
        out = w.apply_generated_unitary(float(gd["t_" + tag]), "chebyshev", ham,
                                        accuracy=1e-13, expansion=200,
                                        spec_lim=list(gd["lim_" + tag]))
        got = out.get_coeff((na + nb, na - nb)).cpu().numpy()
        assert numpy.abs(got - gd[key]).max() < 1e-12
