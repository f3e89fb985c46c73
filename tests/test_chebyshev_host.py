"""The Chebyshev propagator's host loop (fqe_gb300.wavefunction.
chebyshev_series, the branch of apply_generated_unitary at
wavefunction.py:570-606) on the CPU: run over numpy-backed stand-ins of the
Wavefunction vector operations with the oracle's apply as H, against the
reference's own outputs (tests/golden/chebyshev.npz)."""

import copy

import numpy
import pytest


class _Vec:
    """scale / ax_plus_y / norm / deepcopy, as Wavefunction has them."""

    def __init__(self, a):
        self.a = numpy.array(a, dtype=numpy.complex128)

    def scale(self, s):
        self.a *= s

    def ax_plus_y(self, s, other):
        self.a += s * other.a

    def norm(self):
        return float(numpy.linalg.norm(self.a))

    def __deepcopy__(self, memo):
        return _Vec(self.a.copy())


def test_chebyshev_series_matches_reference(golden, oracle):
    from fqe_gb300.wavefunction import chebyshev_series
    gd = golden("chebyshev")
    for key in [k for k in gd if k.startswith("out_")]:
        tag = key[4:]
        norb, na, nb = map(int, tag.split("_"))
        g = oracle.graph(norb, na, nb)
        tensors = (gd["h1_" + tag], gd["h2_" + tag])
        e0 = complex(gd["e0_" + tag])

        def apply_h(v):
            return _Vec(oracle.apply_restricted(v.a, tensors, e0, g))
        out = chebyshev_series(_Vec(gd["psi_" + tag]), apply_h, float(gd["t_" + tag]),
                               1e-13, 200, list(gd["lim_" + tag]), e0)
        assert numpy.abs(out.a - gd[key]).max() < 1e-12


def test_chebyshev_series_expansion_limit(oracle):
    from fqe_gb300.wavefunction import chebyshev_series
    g = oracle.graph(3, 1, 1)
    psi = numpy.ones((3, 3)) / 3.0
    h1 = numpy.diag([1.0, 2.0, 3.0])

    def apply_h(v):
        return _Vec(oracle.apply_restricted(v.a, (h1,), 0.0, g))
    with pytest.raises(RuntimeError, match="chebyshev"):
        chebyshev_series(_Vec(psi), apply_h, 5.0, 1e-15, 3, [0.0, 7.0], 0.0)
