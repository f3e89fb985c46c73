"""Host-side pieces of the learned preconditioner (fqe_gb300/precond.py) on
the CPU: the MINRES solver that produces the training targets (with its
vector kernels replaced inside this test by torch CPU operations), the
parameter initialisation and the diagonal statistics.  The device kernels
are checked against oracle/mlp_oracle.py in tests/test_gpu_mlp.py."""

import numpy
import pytest
import torch


@pytest.fixture
def cpu_vector_ops(monkeypatch):
    from fqe_gb300 import precond

    def vdot(x, y):
        return complex(torch.vdot(x.reshape(-1), y.reshape(-1)))

    def axpy(a, x, y):
        y += complex(a) * x

    def scale(a, x):
        x *= complex(a)

    def norm(x):
        return float(torch.linalg.norm(x))

    for name, fn in (("_vdot", vdot), ("_axpy", axpy), ("_scale", scale),
                     ("_norm", norm)):
        monkeypatch.setattr(precond, name, fn)
    return precond


@pytest.mark.parametrize("shift", [0.0, 0.37])
def test_minres_solves_hermitian_indefinite_systems(cpu_vector_ops, shift):
    # the Jacobi-Davidson correction operator (H - theta) is indefinite
    precond = cpu_vector_ops
    rng = numpy.random.default_rng(1)
    n = 60
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    H = 0.5 * (a + a.conj().T)
    w = numpy.linalg.eigvalsh(H)
    theta = 0.5 * (w[10] + w[11]) + shift  # inside the spectrum
    A = torch.from_numpy(H - theta * numpy.eye(n))
    b = torch.from_numpy(rng.normal(size=n) + 1j * rng.normal(size=n))
    x, rel, its = precond.minres(lambda v: A @ v, b, tol=1e-12, maxiter=400)
    want = numpy.linalg.solve(A.numpy(), b.numpy())
    assert numpy.linalg.norm(x.numpy() - want) / numpy.linalg.norm(want) < 1e-8
    assert rel < 1e-12 and 0 < its <= 400
    # the returned estimate tracks the true residual
    true_rel = float(torch.linalg.norm(A @ x - b) / torch.linalg.norm(b))
    assert true_rel < 1e-10


def test_minres_zero_right_hand_side(cpu_vector_ops):
    precond = cpu_vector_ops
    b = torch.zeros(8, dtype=torch.complex128)
    x, rel, its = precond.minres(lambda v: 2 * v, b)
    assert its == 0 and rel == 0.0 and float(torch.linalg.norm(x)) == 0.0


def test_initial_parameters_are_the_plain_preconditioner():
    from fqe_gb300 import precond
    import mlp_oracle
    p = precond.init_params(0)
    assert p.dtype == numpy.float32 and p.size == mlp_oracle.NPARAM
    # zero output layer: z = 0 for any features, so m = 1 + tanh(0) = 1
    f = numpy.random.default_rng(0).normal(size=(5, 34))
    numpy.testing.assert_allclose(mlp_oracle.forward(p, f), 1.0, atol=0)


def test_diagonal_statistics_use_the_population_deviation():
    from fqe_gb300.precond import _diag_stats
    d = torch.tensor([1.0, 2.0, 4.0, 7.0], dtype=torch.float64)
    s, m = _diag_stats(d)
    assert s == pytest.approx(numpy.std(d.numpy())) and m == 1.0
