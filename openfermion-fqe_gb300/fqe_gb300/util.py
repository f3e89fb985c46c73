"""Helpers of fqe/util.py used on the path."""

from typing import Tuple


def alpha_beta_electrons(nele: int, m_s: int) -> Tuple[int, int]:
    """(nalpha, nbeta) from particle number and spin projection
    (util.py:29-51)."""
    if nele < 0:
        raise ValueError("Cannot have negative electrons")
    if nele < abs(m_s):
        raise ValueError("Spin quantum number exceeds physical limits")
    if (nele + m_s) % 2 != 0:
        raise ValueError("Parity of spin quantum number and number of "
                         "electrons is incompatible")
    nalpha = int(nele + m_s) // 2
    nbeta = nele - nalpha
    return nalpha, nbeta


def validate_config(nalpha: int, nbeta: int, norb: int) -> None:
    """util.py:440-463."""
    if nalpha < 0 or nbeta < 0:
        raise ValueError("Cannot have negative electrons")
    if nalpha > norb or nbeta > norb:
        raise ValueError("Number of electrons exceeds the number of orbitals")


def vdot(wfn1, wfn2) -> complex:
    """<wfn1|wfn2> with conjugation on wfn1, over common sectors
    (util.py:506-530)."""
    ipval = 0.0 + 0.0j
    for key in wfn1.sectors():
        if key in wfn2.sectors():
            ipval += wfn1._civec[key].vdot(wfn2._civec[key])
    return ipval
