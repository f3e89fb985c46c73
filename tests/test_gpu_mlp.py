"""The learned preconditioner's CUDA kernels (csrc/mlp.cu) against the CPU
FP64 oracle (oracle/mlp_oracle.py): features + forward, fused
preconditioning, loss and gradient, gradient accumulation, Adam; and the
training loop on correction-equation samples produced by the GPU Davidson."""

import numpy
import pytest

import mlp_oracle as mo

pytestmark = pytest.mark.gpu

FWD_TOL = 2e-5     # float32 network vs float64 oracle, same bf16 weights
GRAD_TOL = 2e-4    # relative 2-norm of the gradient difference


def _params(seed, out_scale=0.3):
    rng = numpy.random.default_rng(seed)
    p = mo.init_params(seed)
    p[-65:] = rng.normal(0.0, out_scale, 65).astype(numpy.float32)
    p[mo.NIN * 64:mo.NIN * 64 + 64] = rng.normal(0.0, 0.1, 64)  # b1
    return p


def _setup(gpu, norb=6, na=3, nb=2, seed=0):
    import torch
    from fqe_gb300.fci_graph import get_graph
    g = get_graph(na, nb, norb)
    rng = numpy.random.default_rng(seed)
    n = g.lena() * g.lenb()
    diag = rng.normal(0.0, 2.0, n)
    theta = float(diag.min() + 0.37)
    f = mo.features(diag, theta, g.string_alpha_all(), g.string_beta_all(),
                    norb, na, nb, diag.std(), diag.min())
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    x /= numpy.linalg.norm(x)
    r = rng.normal(size=n) + 1j * rng.normal(size=n)
    a = rng.normal(size=n) + 1j * rng.normal(size=n)
    a -= x * numpy.vdot(x, a)
    dev = lambda v: torch.from_numpy(numpy.ascontiguousarray(v)).cuda()
    return dict(g=g, n=n, diag=diag, theta=theta, f=f, x=x, r=r, a=a,
                d_diag=dev(diag.reshape(g.lena(), g.lenb())),
                d_x=dev(x.reshape(g.lena(), g.lenb())),
                d_r=dev(r.reshape(g.lena(), g.lenb())),
                d_a=dev(a.reshape(g.lena(), g.lenb())),
                scale=float(diag.std()), emin=float(diag.min()))


@pytest.mark.parametrize("norb,na,nb", [(6, 3, 2), (8, 4, 4), (10, 5, 3),
                                        (16, 1, 1), (4, 0, 2)])
def test_multiplier_matches_oracle(gpu, norb, na, nb):
    from fqe_gb300.precond import LearnedPreconditioner
    s = _setup(gpu, norb, na, nb, seed=norb)
    p = _params(1)
    pre = LearnedPreconditioner(p)
    m = pre.multiplier(s["theta"], s["d_diag"], s["g"]).cpu().numpy().ravel()
    want = mo.forward(p, s["f"])
    numpy.testing.assert_allclose(m, want, rtol=FWD_TOL, atol=FWD_TOL)
    assert m.min() > 0.0 and m.max() < 2.0


def test_precondition_matches_oracle(gpu):
    from fqe_gb300.precond import LearnedPreconditioner
    s = _setup(gpu, 8, 4, 3, seed=3)
    s["d_diag"].view(-1)[:5] = s["theta"]  # floored denominators
    diag = s["d_diag"].cpu().numpy().ravel()
    p = _params(2)
    pre = LearnedPreconditioner(p)
    t = pre(s["d_r"], s["theta"], s["d_diag"], s["g"]).cpu().numpy().ravel()
    f = mo.features(diag, s["theta"], s["g"].string_alpha_all(),
                    s["g"].string_beta_all(), 8, 4, 3, pre.stats(s["d_diag"])[0],
                    pre.stats(s["d_diag"])[1])
    want = mo.precondition(p, s["r"], diag, s["theta"], f, 1e-4)
    numpy.testing.assert_allclose(t, want, rtol=FWD_TOL, atol=0)


def test_zero_network_is_the_plain_preconditioner(gpu):
    import torch
    from fqe_gb300 import _lib
    from fqe_gb300.fqe_data import _ptr, _stream
    from fqe_gb300.precond import LearnedPreconditioner
    s = _setup(gpu, 7, 3, 3, seed=4)
    pre = LearnedPreconditioner()  # all parameters zero: m = 1 exactly
    t = pre(s["d_r"], s["theta"], s["d_diag"], s["g"])
    plain = torch.empty_like(s["d_r"])
    _lib.call("fqegpu_precondition", plain.numel(), _ptr(s["d_r"]),
              _ptr(s["d_diag"]), s["theta"], 1e-4, _ptr(plain), _stream())
    assert torch.equal(t, plain)


def test_loss_and_gradient_match_oracle(gpu):
    import torch
    from fqe_gb300.precond import CorrectionSample, LearnedPreconditioner
    s = _setup(gpu, 8, 4, 4, seed=5)
    diag = s["diag"]
    u = s["r"] / mo.floored(diag, s["theta"], 1e-4)
    p = _params(3)
    pre = LearnedPreconditioner(p)
    sample = CorrectionSample(
        graph=s["g"], diag=s["d_diag"], theta=s["theta"],
        u=torch.from_numpy(u.reshape(s["d_r"].shape)).cuda(), x=s["d_x"],
        a=s["d_a"], scale=s["scale"], emin=s["emin"])
    loss = pre.loss_grad(sample)
    g = pre.grad().astype(numpy.float64)
    L, want = mo.loss_and_grad(p, s["f"], u, s["x"], s["a"])
    assert abs(loss - L) < 1e-6
    assert numpy.linalg.norm(g - want) <= GRAD_TOL * numpy.linalg.norm(want)
    # accumulation: grad(s) + grad(s) = 2 grad(s)
    pre.loss_grad(sample, accumulate=True)
    g2 = pre.grad().astype(numpy.float64)
    numpy.testing.assert_allclose(g2, 2.0 * g, rtol=1e-6, atol=1e-12)


def test_adam_matches_oracle(gpu):
    import torch
    from fqe_gb300.precond import CorrectionSample, LearnedPreconditioner
    s = _setup(gpu, 6, 3, 3, seed=6)
    u = s["r"] / mo.floored(s["diag"], s["theta"], 1e-4)
    p = _params(4)
    pre = LearnedPreconditioner(p)
    sample = CorrectionSample(
        graph=s["g"], diag=s["d_diag"], theta=s["theta"],
        u=torch.from_numpy(u.reshape(s["d_r"].shape)).cuda(), x=s["d_x"],
        a=s["d_a"], scale=s["scale"], emin=s["emin"])
    state = (numpy.zeros(mo.NPARAM), numpy.zeros(mo.NPARAM), 0)
    ref = p.copy()
    for _ in range(3):
        pre.loss_grad(sample)
        g = pre.grad().astype(numpy.float64)
        pre.adam(1e-3, grad_scale=0.5)
        ref, state = mo.adam(ref, 0.5 * g, state, 1e-3)
    numpy.testing.assert_allclose(pre.params(), ref, rtol=1e-5, atol=1e-7)


def test_minres_solves_correction_equation(gpu):
    # the sampler's MINRES against a dense solve of the projected equation
    import torch
    from fqe_gb300 import davidson, precond, synthetic
    from oracle import dense_hamiltonian, graph
    h1, h2, _ = synthetic.integrals(6, 12, 31)
    ham = gpu.RestrictedHamiltonian((h1, h2))
    store = []
    davidson.davidson(ham, 3, 3, max_iter=3,
                      callback=precond.correction_sampler(store, tol=1e-12,
                                                          maxiter=2000))
    assert len(store) == 3
    H = dense_hamiltonian(h1.astype(complex), h2.astype(complex), graph(6, 3, 3))
    for smp in store:
        x = smp.x.cpu().numpy().ravel()
        a = smp.a.cpu().numpy().ravel()
        P = numpy.eye(len(x)) - numpy.outer(x, x.conj())
        A = P @ (H - smp.theta * numpy.eye(len(x))) @ P
        r = (H @ x) - smp.theta * x
        assert abs(numpy.vdot(x, a)) < 1e-10
        assert numpy.linalg.norm(A @ a + r) < 1e-8 * numpy.linalg.norm(r)


def test_training_reduces_loss(gpu):
    # hand-written forward/backward + Adam on samples the GPU Davidson
    # produces: the training loss goes down from the plain preconditioner's
    from fqe_gb300 import davidson, precond, synthetic
    samples = []
    for seed in (41, 42):
        h1, h2, _ = synthetic.integrals(8, 16, seed)
        ham = gpu.RestrictedHamiltonian((h1, h2))
        davidson.davidson(ham, 4, 4, max_iter=8,
                          callback=precond.correction_sampler(samples))
    pre = precond.LearnedPreconditioner(precond.init_params(0))
    plain = precond.mean_loss(pre, samples)
    hist = precond.train(pre, samples, epochs=15, lr=2e-3, batch=2)
    assert hist[-1] < plain
    assert precond.mean_loss(pre, samples) < plain


def test_trained_network_gain(gpu):
    # What the shipped network (trained on norb 10-12 correction equations,
    # fqe_gb300/data/precond_mlp.npz) gains over the plain preconditioner on
    # held-out sectors: a lower correction-equation loss, the objective it was
    # trained on.  Davidson with it, watched by the residual guard with the plain
    # fallback, converges to the plain run's energy; the iteration counts are
    # printed, not asserted (on these synthetic integrals the learned
    # multiplier costs iterations).
    from fqe_gb300 import davidson, precond, synthetic
    pre = precond.LearnedPreconditioner.load()
    plain = precond.LearnedPreconditioner()
    samples = []
    for seed in (3000, 3001):
        h1, h2, _ = synthetic.integrals(10, 20, seed)
        ham = gpu.RestrictedHamiltonian((h1, h2))
        davidson.davidson(ham, 5, 5, block=4, max_iter=24,
                          callback=precond.correction_sampler(
                              samples, every=3, tol=1e-6, maxiter=200))
    loss_plain = precond.mean_loss(plain, samples)
    loss_learned = precond.mean_loss(pre, samples)
    h1, h2, _ = synthetic.integrals(10, 20, 3000)
    ham = gpu.RestrictedHamiltonian((h1, h2))
    r_plain = davidson.davidson(ham, 5, 5, block=4)
    r_learned = davidson.davidson(ham, 5, 5, block=4, preconditioner=pre,
                                  max_iter=400)
    print(f"held-out correction-equation loss: plain {loss_plain:.4f}, "
          f"learned {loss_learned:.4f}; Davidson iterations: plain "
          f"{r_plain.iterations}, learned {r_learned.iterations} (plain "
          f"fallback at {r_learned.fallback_iteration})")
    assert loss_learned < loss_plain
    assert r_plain.converged and r_learned.converged
    assert abs(r_plain.eigenvalues[0] - r_learned.eigenvalues[0]) < 1e-9
