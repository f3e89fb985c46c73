"""fqe_gb300 — the restricted H·psi path of OpenFermion-FQE on one GB300.

Public names follow the reference package ``fqe`` (fqe/__init__.py and
_fqe_control.py): Wavefunction, FqeData, FciGraph, RestrictedHamiltonian,
DiagonalCoulomb, get_wavefunction, get_restricted_hamiltonian,
get_diagonalcoulomb_hamiltonian, apply, time_evolve, expectationValue, vdot.
All arithmetic runs in libfqegpu.so (hand-written sm_103a CUDA).
"""

from . import settings
from .fci_graph import FciGraph
from .fqe_data import FqeData
from .hamiltonians import (DiagonalCoulomb, General, Hamiltonian, RestrictedHamiltonian,
                           build_hamiltonian)
from .util import alpha_beta_electrons, vdot
from .wavefunction import Wavefunction


def get_wavefunction(nele: int, m_s: int, norb: int) -> Wavefunction:
    """_fqe_control.py get_wavefunction."""
    return Wavefunction([[nele, m_s, norb]])


def get_number_conserving_wavefunction(nele: int, norb: int) -> Wavefunction:
    param = []
    maxalpha = min(norb, nele)
    minalpha = nele - maxalpha
    for nalpha in range(minalpha, maxalpha + 1):
        nbeta = nele - nalpha
        if nbeta <= norb:
            param.append([nele, nalpha - nbeta, norb])
    return Wavefunction(param)


def get_restricted_hamiltonian(tensors, e_0: complex = 0. + 0.j
                               ) -> RestrictedHamiltonian:
    """_fqe_control.py:559-576."""
    return RestrictedHamiltonian(tensors, e_0=e_0)


def get_diagonalcoulomb_hamiltonian(h2e, e_0: complex = 0. + 0.j
                                    ) -> DiagonalCoulomb:
    """_fqe_control.py:495-508."""
    return DiagonalCoulomb(h2e, e_0=e_0)


def apply(ops, wfn: Wavefunction) -> Wavefunction:
    """_fqe_control.py:356-371."""
    return wfn.apply(ops)


def time_evolve(wfn: Wavefunction, time: float, hamil,
                inplace: bool = False) -> Wavefunction:
    """_fqe_control.py:180-198."""
    return wfn.time_evolve(time, hamil, inplace)


def expectationValue(wfn: Wavefunction, ops, brawfn=None) -> complex:
    return wfn.expectationValue(ops, brawfn)


def build() -> str:
    """Compile libfqegpu.so in-tree (nvcc, sm_103a)."""
    from ._build import build as _b
    return _b()
