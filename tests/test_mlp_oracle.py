"""The CPU FP64 oracle of the learned preconditioner (oracle/mlp_oracle.py):
its analytic gradient against central finite differences, its feature
encoding against hand-worked strings, bf16 rounding against known values."""

import numpy
import pytest

import mlp_oracle as mo


def _sample(oracle, norb=5, na=2, nb=2, seed=0):
    rng = numpy.random.default_rng(seed)
    g = oracle.graph(norb, na, nb)
    n = g.lena * g.lenb
    diag = rng.normal(0.0, 2.0, n)
    theta = diag.min() + 0.3
    f = mo.features(diag, theta, g.astr, g.bstr, norb, na, nb,
                    diag.std(), diag.min())
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    x /= numpy.linalg.norm(x)
    r = rng.normal(size=n) + 1j * rng.normal(size=n)
    a = rng.normal(size=n) + 1j * rng.normal(size=n)
    a -= x * numpy.vdot(x, a)
    u = r / mo.floored(diag, theta, 1e-4)
    return f, u, x, a


def test_bf16_rounding_known_values():
    v = numpy.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-9, -3.14159265, 1e-3],
                    dtype=numpy.float32)
    got = mo.bf16_round(v)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to even (1.0);
    # 1 + 3*2^-9 rounds up to 1 + 2^-7
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == numpy.float32(1 + 2**-7)
    assert got[3] == numpy.float32(-3.140625)
    assert abs(got[4] - 1e-3) / 1e-3 < 2**-8


def test_feature_slots():
    # norb 6, 2 alpha electrons: slot k <-> orbital k - 6; slots 0..5 are the
    # filled core, slots 6..11 orbitals 0..5, slots 12..15 empty
    b = mo.slot_bits([0b000011, 0b100100], 6, 2)
    assert list(b[0]) == [1] * 6 + [1, 1, 0, 0, 0, 0] + [0] * 4
    assert list(b[1]) == [1] * 6 + [0, 0, 1, 0, 0, 1] + [0] * 4
    # norb 16 with 8 electrons: slot k is orbital k
    s = 0b1010000000001111
    assert list(mo.slot_bits([s], 16, 8)[0]) == [(s >> k) & 1 for k in range(16)]
    # 10 electrons in 16 orbitals: slot k is orbital k + 2 (orbitals 0, 1 dropped)
    s = 0b0000001111111111
    assert list(mo.slot_bits([s], 16, 10)[0]) == [(s >> (k + 2)) & 1 for k in range(16)]


def test_gradient_finite_differences(oracle):
    f, u, x, a = _sample(oracle)
    rng = numpy.random.default_rng(1)
    p = mo.init_params(3).astype(numpy.float64)
    p[-65:] = rng.normal(0.0, 0.3, 65)  # non-zero output layer
    L, g = mo.loss_and_grad(p, f, u, x, a, rounding=False)
    assert 0.0 <= L <= 1.0
    idx = numpy.concatenate([rng.choice(mo.NPARAM - 65, 40, replace=False),
                             numpy.arange(mo.NPARAM - 65, mo.NPARAM, 7)])
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mo.loss_and_grad(pp, f, u, x, a, rounding=False)[0]
              - mo.loss_and_grad(pm, f, u, x, a, rounding=False)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-8, (k, fd, g[k])


def test_loss_invariances(oracle):
    f, u, x, a = _sample(oracle, seed=2)
    m = 1.0 + 0.5 * numpy.tanh(numpy.random.default_rng(0).normal(size=len(u)))
    L1, d1 = mo.loss_and_dm(m, u, x, a)
    L2, d2 = mo.loss_and_dm(3.0 * m, u, x, a)      # scale invariant
    assert abs(L1 - L2) < 1e-12
    L3, _ = mo.loss_and_dm(m, u, x, (2 - 1j) * a)  # target phase/scale
    assert abs(L1 - L3) < 1e-12
    # m * u == a (+ any multiple of x) gives zero loss
    mm = numpy.ones(len(u))
    L0, _ = mo.loss_and_dm(mm, a + 0.7 * x, x, a)
    assert L0 < 1e-14
