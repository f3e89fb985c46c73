"""Host logic of the block Davidson driver (fqe_gb300/davidson.py) on the CPU:
the projected problem, block Gram-Schmidt, restarts, the residual stopping
rule, several roots and the learned-preconditioner guard, with the sector's
operator and the vector kernels replaced inside this test by dense CPU
stand-ins (the oracle's dense H of a small sector; torch CPU vector ops).
The GPU runs of the same driver are in tests/test_gpu_davidson.py."""

import numpy
import pytest
import torch


class _DenseOperator:
    """Stands in for davidson._Operator: H of one small sector as a dense
    matrix (built by the oracle), applied on CPU tensors."""

    def __init__(self, H, shape):
        self.H = torch.from_numpy(H)
        self.shape = shape
        self.diag = torch.from_numpy(numpy.real(numpy.diag(H)).copy()).reshape(shape)
        self.graph = None
        self.applies = 0

    def apply(self, v):
        self.applies += 1
        return (self.H @ v.reshape(-1)).reshape(self.shape)

    def check(self):  # no device waits on the CPU
        pass


def _plain(r, theta, diag, graph, floor=1e-4):
    d = theta - diag
    d = torch.where(d.abs() < floor, torch.full_like(d, floor) * torch.sign(d + 1e-300), d)
    return r / d


class _Learned:
    """A preconditioner with a `plain` method whose own correction is poor
    (r itself): the residual guard must switch to the plain one."""

    def __init__(self):
        self.calls = 0

    def __call__(self, r, theta, diag, graph):
        self.calls += 1
        return r.clone()

    def plain(self, r, theta, diag, graph):
        return _plain(r, theta, diag, graph)


@pytest.fixture
def dense_davidson(monkeypatch, oracle):
    from fqe_gb300 import davidson as dav
    from fqe_gb300 import synthetic

    def vdot(x, y):
        return complex(torch.vdot(x.reshape(-1), y.reshape(-1)))

    def axpy(a, x, y):
        y += complex(a) * x

    def norm(x):
        return float(torch.linalg.norm(x))

    def block_vdot(vs, t):
        return numpy.array([vdot(v, t) for v in vs])

    def block_axpy(coef, vs, t):
        for c, v in zip(numpy.asarray(coef), vs):
            t += complex(c) * v

    def scale(a, x):
        x *= complex(a)

    for name, fn in (("_vdot", vdot), ("_axpy", axpy), ("_norm", norm),
                     ("_block_vdot", block_vdot), ("_block_axpy", block_axpy),
                     ("_scale", scale)):
        monkeypatch.setattr(dav, name, fn)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)

    def make(norb, na, nb, seed):
        h1, h2, _ = synthetic.sector(norb, na, nb, 2 * norb, seed)
        g = oracle.graph(norb, na, nb)
        H = oracle.dense_hamiltonian(h1, h2, g)
        H = 0.5 * (H + H.conj().T)
        op = _DenseOperator(H, (g.lena, g.lenb))
        monkeypatch.setattr(dav, "_Operator", lambda *a, **k: op)
        return dav, op, numpy.linalg.eigvalsh(H)

    return make


def test_lowest_root_and_restart(dense_davidson):
    dav, op, w = dense_davidson(5, 2, 2, 1)
    r = dav.davidson(None, 2, 2, block=2, tol=1e-9, max_subspace=6,
                     max_iter=300, preconditioner=_plain)
    assert r.converged
    assert abs(r.eigenvalues[0] - w[0]) < 1e-12
    x = r.vectors[0].reshape(-1)
    assert abs(float(torch.linalg.norm(x)) - 1.0) < 1e-12
    res = op.H @ x - w[0] * x
    assert float(torch.linalg.norm(res)) < 1e-8
    # a six-vector subspace with blocks of two restarts many times
    assert r.iterations > 3 and r.applies == op.applies


def test_several_roots(dense_davidson):
    dav, op, w = dense_davidson(5, 3, 1, 2)
    r = dav.davidson(None, 3, 1, nroots=3, block=3, tol=1e-8, max_subspace=24,
                     max_iter=300, preconditioner=_plain)
    assert r.converged
    numpy.testing.assert_allclose(r.eigenvalues, w[:3], atol=1e-11)
    # Ritz vectors orthonormal
    X = torch.stack([v.reshape(-1) for v in r.vectors])
    numpy.testing.assert_allclose((X.conj() @ X.T).numpy(), numpy.eye(3), atol=1e-10)


def test_residual_guard_switches_to_plain(dense_davidson):
    dav, op, w = dense_davidson(5, 2, 2, 3)
    pre = _Learned()
    r = dav.davidson(None, 2, 2, block=1, tol=1e-8, max_subspace=12,
                     max_iter=400, preconditioner=pre, patience=4)
    assert r.converged and abs(r.eigenvalues[0] - w[0]) < 1e-11
    assert r.fallback_iteration is not None
    assert pre.calls >= 1


def test_bad_arguments(dense_davidson):
    dav, op, w = dense_davidson(4, 2, 1, 4)
    with pytest.raises(ValueError):
        dav.davidson(None, 2, 1, block=4, max_subspace=6)
    n = op.shape[0] * op.shape[1]
    with pytest.raises(ValueError, match="Number of roots"):
        dav.davidson(None, 2, 1, nroots=n + 1, max_subspace=2 * n + 2)
