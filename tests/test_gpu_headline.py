"""Parity at the benchmarked configuration.

* The H*psi workload of bench.py: the norb=14 (7a,7b) sector, 11,778,624
  determinants, seeded synthetic integrals with 28 Cholesky vectors, seed 0
  (fqe_gb300.synthetic.sector).  The FP64 GPU apply and the tensor-core
  (Ozaki-split BF16) apply are compared with the oracle's apply
  (the reference's C algorithm restated, oracle/fqe_oracle.c) on the same
  inputs: relative 2-norm error <= 1e-12 (FP64) and <= 1e-10 (tensor cores),
  the tolerances of _apply_array_spatial12_lm's complex128 path
  (fqe_data.py:685-710) that the library promises.
* The Taylor step of the benchmark's norb-14 configuration (t = 0.05 to
  1e-12): tensor-core against FP64, <= 1e-10, norms kept to 1e-12.
* The norb=16 (8a,8b) sector (165,636,900 determinants, 32 Cholesky vectors):
  too large for the CPU oracle, so the validated FP64 GPU apply is the
  reference of the tensor-core apply (<= 1e-10).
"""

import os

import numpy
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_OZ = 1e-10


def _rel(a, b):
    return float(numpy.linalg.norm(a - b) / numpy.linalg.norm(b))


@pytest.fixture(scope="module")
def headline(oracle):
    from fqe_gb300 import synthetic
    h1, h2, psi = synthetic.sector(14, 7, 7, 28, 0)
    oracle.set_threads(os.cpu_count() or 1)
    g = oracle.graph(14, 7, 7)
    want = oracle.apply_spatial12(psi, h1, h2, g)
    return h1, h2, psi, want


def _apply(gpu, h1, h2, psi, precision):
    import torch
    from fqe_gb300 import settings
    from fqe_gb300.fqe_data import check_apply, ham_for
    d = gpu.FqeData(7, 7, 14)
    d.set_wfn(strategy="from_data", raw_data=psi)
    old = settings.precision
    settings.precision = precision
    try:
        ham = ham_for(d._core, h1, h2)
        out = d._run_apply(ham)
        check_apply(ham)
        torch.cuda.synchronize()
        return out.cpu().numpy()
    finally:
        settings.precision = old


def test_headline_fp64_matches_oracle(gpu, headline):
    h1, h2, psi, want = headline
    err = _rel(_apply(gpu, h1, h2, psi, "fp64"), want)
    print(f"norb 14 FP64 apply vs oracle: {err:.3e}")
    assert err < TOL_FP64


def test_headline_tensor_core_matches_oracle(gpu, headline):
    h1, h2, psi, want = headline
    err = _rel(_apply(gpu, h1, h2, psi, "ozaki"), want)
    print(f"norb 14 tensor-core apply vs oracle: {err:.3e}")
    assert err < TOL_OZ


def test_headline_taylor_step(gpu):
    from fqe_gb300 import settings, synthetic
    h1, h2, psi = synthetic.sector(14, 7, 7, 28, 0)
    ham = gpu.RestrictedHamiltonian((h1, h2))
    out = {}
    old = settings.precision
    try:
        for prec in ("fp64", "ozaki"):
            settings.precision = prec
            w = gpu.Wavefunction([[14, 0, 14]])
            w.set_wfn(strategy="from_data", raw_data={(14, 0): psi})
            ev = w.apply_generated_unitary(0.05, "taylor", ham, accuracy=1e-12,
                                           expansion=80)
            out[prec] = ev.get_coeff((14, 0)).cpu().numpy()
    finally:
        settings.precision = old
    err = _rel(out["ozaki"], out["fp64"])
    print(f"norb 14 Taylor t=0.05: tensor-core vs FP64 {err:.3e}")
    assert err < TOL_OZ
    for prec in out:
        assert abs(numpy.linalg.norm(out[prec]) - 1.0) < 1e-12


def test_norb16_tensor_core_matches_fp64(gpu):
    import torch
    from fqe_gb300 import settings, synthetic
    from fqe_gb300.fqe_data import check_apply, ham_for
    h1, h2 = synthetic.integrals(16, 32, 0)[:2]
    d = gpu.FqeData(8, 8, 16)
    gen = torch.Generator(device="cuda").manual_seed(0)
    psi = torch.complex(torch.randn(d.coeff.shape, dtype=torch.float64, device="cuda",
                                    generator=gen),
                        torch.randn(d.coeff.shape, dtype=torch.float64, device="cuda",
                                    generator=gen))
    psi /= torch.linalg.norm(psi)
    d.coeff.copy_(psi)
    ham = ham_for(d._core, h1, h2)
    res = {}
    old = settings.precision
    try:
        for prec in ("fp64", "ozaki"):
            settings.precision = prec
            res[prec] = d._run_apply(ham)
            check_apply(ham)
    finally:
        settings.precision = old
    err = float(torch.linalg.norm(res["ozaki"] - res["fp64"]) /
                torch.linalg.norm(res["fp64"]))
    print(f"norb 16 (8,8) tensor-core vs FP64 GPU apply: {err:.3e}")
    assert err < TOL_OZ


def test_twenty_taylor_steps_norm_and_fidelity(gpu):
    """The 20-step evolution of the benchmark's norb-16 configuration (dt =
    0.05, accuracy 1e-12, Wavefunction.apply_generated_unitary 'taylor',
    wavefunction.py:553-568), at norb 12 (6a,6b) so that the FP64 path can
    follow every step: on the tensor cores the norm stays within 1e-9 of 1
    over the 20 steps, the first step's fidelity |<psi_oz|psi_fp64>|^2 is
    within 1e-10 of 1 and its relative difference below 1e-10, and after 20
    steps the two trajectories still agree to 1e-9."""
    import torch
    from fqe_gb300 import settings, synthetic
    norb, na, nb = 12, 6, 6
    h1, h2, psi = synthetic.sector(norb, na, nb, synthetic.default_nchol(norb), 0)
    ham = gpu.RestrictedHamiltonian((h1, h2))
    key = (na + nb, na - nb)
    old = settings.precision
    traj = {}
    try:
        for prec in ("ozaki", "fp64"):
            settings.precision = prec
            w = gpu.Wavefunction([[na + nb, na - nb, norb]])
            w.set_wfn(strategy="from_data", raw_data={key: psi})
            states = []
            for _ in range(20):
                w = w.apply_generated_unitary(0.05, "taylor", ham, accuracy=1e-12,
                                              expansion=80)
                states.append(w.get_coeff(key).clone())
            traj[prec] = states
    finally:
        settings.precision = old
    oz, f64 = traj["ozaki"], traj["fp64"]
    for s in oz:
        assert abs(float(torch.linalg.norm(s)) - 1.0) < 1e-9
    a, b = oz[0].reshape(-1), f64[0].reshape(-1)
    fid = abs(complex(torch.vdot(a, b))) ** 2 / (float(torch.linalg.norm(a)) ** 2 *
                                                 float(torch.linalg.norm(b)) ** 2)
    assert 1.0 - fid < 1e-10
    assert float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) < 1e-10
    assert float(torch.linalg.norm(oz[-1] - f64[-1]) / torch.linalg.norm(f64[-1])) < 1e-9
