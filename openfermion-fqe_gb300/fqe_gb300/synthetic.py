"""Seeded synthetic sectors for tests and benchmarks.

The integral generator draws, from numpy.random.default_rng(seed), in order:
  h1  = N(0,1) * exp(-|i-j|/2), symmetrised (A + A^T)/2;
  L_t ~ N(0, 0.3) for t < T, each symmetrised;
  (ij|kl) = sum_t L_t[i,j] L_t[k,l]   (chemist notation, 8-fold symmetric, PSD);
  h2 = -0.5 * einsum('ikjl->ijkl', eri)  (the FQE restricted convention:
       h2[i,j,k,l] multiplies sum_{s,t} a+_is a+_jt a_ks a_lt, i.e. -1/2 (ik|jl));
  psi = N(0,1) + i N(0,1), normalised;
  V (diagonal Coulomb) ~ N(0, 0.5), symmetrised.
T is 16, 28, 32 for norb 8, 14, 16 (norb // 2 + 2 * (norb // 2) otherwise is
not used: callers pass T).
"""

import math

import numpy


def integrals(norb: int, nchol: int, seed: int = 0):
    rng = numpy.random.default_rng(seed)
    idx = numpy.arange(norb)
    h1 = rng.standard_normal((norb, norb)) * numpy.exp(
        -numpy.abs(idx[:, None] - idx[None, :]) / 2.0)
    h1 = 0.5 * (h1 + h1.T)
    L = rng.normal(0.0, 0.3, size=(nchol, norb, norb))
    L = 0.5 * (L + numpy.transpose(L, (0, 2, 1)))
    eri = numpy.einsum('tij,tkl->ijkl', L, L)
    h2 = -0.5 * numpy.einsum('ikjl->ijkl', eri)
    return h1, numpy.ascontiguousarray(h2), rng


def wavefunction_coeff(lena: int, lenb: int, rng) -> numpy.ndarray:
    c = rng.standard_normal((lena, lenb)) + 1.0j * rng.standard_normal(
        (lena, lenb))
    return c / numpy.linalg.norm(c)


def sector(norb: int, nalpha: int, nbeta: int, nchol: int, seed: int = 0):
    """(h1, h2, psi) of one seeded sector."""
    h1, h2, rng = integrals(norb, nchol, seed)
    psi = wavefunction_coeff(math.comb(norb, nalpha), math.comb(norb, nbeta),
                             rng)
    return h1, h2, psi


def diagonal_coulomb(norb: int, seed: int = 0) -> numpy.ndarray:
    rng = numpy.random.default_rng(seed + 7919)
    v = rng.normal(0.0, 0.5, size=(norb, norb))
    return 0.5 * (v + v.T)


def default_nchol(norb: int) -> int:
    return {8: 16, 14: 28, 16: 32}.get(norb, 2 * norb)
