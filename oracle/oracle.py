"""ORACLE — test infrastructure only (never imported by the GPU product).

Python side of the CPU restatement of the reference FQE H·psi path.  The
arithmetic lives in ``fqe_oracle.c`` (compiled by ``make -C oracle`` into
``oracle/_build/libfqe_oracle.so``); this module adds the numpy glue that the
reference keeps in Python:

* ``graph``                       FciGraph tables (fci_graph.py:108-154)
* ``prep_spatial12``              h1'/h2' preparation (fqe_data.py:691-693)
* ``apply_spatial12``             _apply_array_spatial12_lm (fqe_data.py:685-710)
* ``apply_spatial1``              dense_apply_array_spatial1 (fqe_data.py:497-526)
* ``apply_spin1`` / ``apply_spin12``  spin-orbital operators (fqe_data.py:533-563,
                                  743-773): the same kernels with spin blocks
* ``transform_orbitals``          an orbital map on a sector through compound
                                  matrices (the result of Wavefunction.transform,
                                  wavefunction.py:813-959, by another route)
* ``apply_restricted``            Wavefunction._apply_array (wavefunction.py:366-399)
* ``taylor_evolve``               apply_generated_unitary, Taylor branch
                                  (wavefunction.py:553-568, 605-606)
* ``chebyshev_evolve``            the same, Chebyshev branch (:570-606)
* ``evolve_diagonal_coulomb`` / ``apply_diagonal_coulomb``
                                  fqe_data.py:263-361 -> lib/fqe_data.c:455-602
* ``make_dvec`` / ``make_coeff``  fqe_data.py:2209-2234, 2309-2334
* ``rdm1``                        FqeData.rdm1 / _rdm1_blocked (fqe_data.py:1668-1724):
                                  rdm1[i][j] = <bra|E_ij|ket> through make_dvec
* ``rdm12``                       FqeData.rdm12, half-filling form (fqe_data.py:1762-1838)
* ``diagonal_energies``           <I|H|I> for a restricted Hamiltonian, by
                                  applying H to unit vectors (small cases only)

``ozaki_model.py`` beside it models this project's tensor-core contraction
arithmetic in numpy (no reference counterpart) for tests/test_ozaki_model.py.

Used by tests/ (the results of the CUDA library are compared with it), by
``__graft_entry__.smoke`` and by
bench.py's CPU legs.  Its parity with the reference is pinned by
tests/test_oracle_pins.py.
"""

import ctypes
import math
import os
import subprocess

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfqe_oracle.so")

_lib = None


def build() -> str:
    """Compile the C restatement (idempotent) and return the library path."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        for name, args in {
                "orc_set_threads": [I],
                "orc_z_matrix": [I, I, P],
                "orc_strings": [I, I, P, P],
                "orc_map_lengths": [I, I, P, P],
                "orc_build_maps": [I, I, I, P, P, P],
                "orc_dexc": [I, I, I, P, P, P],
                "orc_apply12_same_spin": [P, P, P, I, I, I, P, P, I, I],
                "orc_apply12_diff_spin": [P, P, P, P, I, I, I, I, P, I],
                "orc_apply1": [P, P, P, I, I, I, P, I],
                "orc_diagonal_coulomb": [P, P, P, P, P, I, I, I],
                "orc_diagonal_coulomb_apply": [P, P, P, P, P, I, I, I],
                "orc_make_dvec": [P, P, I, P, P, I, I, I],
                "orc_make_coeff": [P, P, I, P, P, I, I, I],
        }.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = I
        L.orc_binomial.argtypes = [I, I]
        L.orc_binomial.restype = ctypes.c_int64
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def set_threads(n: int) -> int:
    return lib().orc_set_threads(int(n))


def z_matrix(norb: int, nele: int) -> numpy.ndarray:
    Z = numpy.zeros((nele, norb), dtype=numpy.int32)
    if Z.size:
        _check(lib().orc_z_matrix(norb, nele, _p(Z)), "z_matrix")
    return Z


def strings(norb: int, nele: int) -> numpy.ndarray:
    n = math.comb(norb, nele)
    out = numpy.zeros(n, dtype=numpy.uint64)
    Z = z_matrix(norb, nele)
    Zc = Z if Z.size else numpy.zeros(1, dtype=numpy.int32)
    _check(lib().orc_strings(norb, nele, _p(Zc), _p(out)), "strings")
    return out


class Graph:
    """String tables of one spin sector pair, as FciGraph holds them."""

    def __init__(self, norb: int, nalpha: int, nbeta: int):
        self.norb, self.nalpha, self.nbeta = norb, nalpha, nbeta
        self.lena = math.comb(norb, nalpha)
        self.lenb = math.comb(norb, nbeta)
        self.astr, self.alens, self.amaps, self.dexca = _spin_tables(
            norb, nalpha)
        self.bstr, self.blens, self.bmaps, self.dexcb = _spin_tables(
            norb, nbeta)

    def alpha_map(self, i, j):
        return _map_slice(self.alens, self.amaps, self.norb, i, j)

    def beta_map(self, i, j):
        return _map_slice(self.blens, self.bmaps, self.norb, i, j)


def _map_slice(lens, maps, norb, i, j):
    off = int(lens.ravel()[:i * norb + j].sum())
    n = int(lens.ravel()[i * norb + j])
    return maps[off:off + n]


def _spin_tables(norb, nele):
    L = lib()
    length = math.comb(norb, nele)
    Z = z_matrix(norb, nele)
    Zc = Z if Z.size else numpy.zeros(1, dtype=numpy.int32)
    strs = strings(norb, nele)
    lens = numpy.zeros((norb, norb), dtype=numpy.int32)
    if norb:
        _check(L.orc_map_lengths(norb, length, _p(strs), _p(lens)), "lengths")
    maps = numpy.zeros((max(int(lens.sum()), 1), 3), dtype=numpy.int32)
    if norb:
        _check(L.orc_build_maps(norb, nele, length, _p(strs), _p(Zc), _p(maps)),
               "maps")
    maps = maps[:int(lens.sum())]
    lk = nele * (norb - nele + 1)
    dexc = numpy.zeros((length, lk, 3), dtype=numpy.int32)
    if dexc.size:
        _check(L.orc_dexc(norb, nele, length, _p(lens), _p(maps), _p(dexc)),
               "dexc")
    return strs, lens, numpy.ascontiguousarray(maps), dexc


_graph_cache = {}


def graph(norb: int, nalpha: int, nbeta: int) -> Graph:
    key = (norb, nalpha, nbeta)
    if key not in _graph_cache:
        _graph_cache[key] = Graph(norb, nalpha, nbeta)
    return _graph_cache[key]


def prep_spatial12(h1, h2):
    """h1' = h1 - sum_k h2'[i,k,k,j],  h2'[i,k,j,l] = -h2[i,j,k,l]
    (fqe_data.py:691-693)."""
    h1p = numpy.array(h1, dtype=numpy.complex128, copy=True)
    h2p = numpy.ascontiguousarray(
        numpy.moveaxis(numpy.asarray(h2, dtype=numpy.complex128), 1, 2) * -1.0)
    h1p -= numpy.einsum("ikkj->ij", h2p)
    return numpy.ascontiguousarray(h1p), h2p


def apply_spatial12(coeff, h1, h2, g: Graph):
    """sigma = (h1, h2) applied to one sector (fqe_data.py:685-710)."""
    L = lib()
    norb = g.norb
    h1p, h2p = prep_spatial12(h1, h2)
    coeff = numpy.ascontiguousarray(coeff, dtype=numpy.complex128)
    out = numpy.zeros_like(coeff)
    if coeff.size == 0 or norb == 0:
        return out
    nda = g.dexca.shape[1]
    ndb = g.dexcb.shape[1]
    if nda:
        _check(L.orc_apply12_same_spin(_p(coeff), _p(out), _p(g.dexca), g.lena,
                                       g.lenb, nda, _p(h1p), _p(h2p), norb, 1),
               "same_spin alpha")
    if ndb:
        _check(L.orc_apply12_same_spin(_p(coeff), _p(out), _p(g.dexcb), g.lena,
                                       g.lenb, ndb, _p(h1p), _p(h2p), norb, 0),
               "same_spin beta")
    if nda and ndb:
        h2ab = numpy.ascontiguousarray(h2p +
                                       numpy.einsum("ijkl->klij", h2p))
        _check(L.orc_apply12_diff_spin(_p(coeff), _p(out), _p(g.dexca),
                                       _p(g.dexcb), g.lena, g.lenb, nda, ndb,
                                       _p(h2ab), norb), "diff_spin")
    return out


def apply_spatial1(coeff, h1, g: Graph):
    """sigma = sum_ij h1_ij E_ij coeff (fqe_data.py:497-526)."""
    L = lib()
    h1c = numpy.ascontiguousarray(h1, dtype=numpy.complex128)
    coeff = numpy.ascontiguousarray(coeff, dtype=numpy.complex128)
    out = numpy.zeros_like(coeff)
    for is_alpha, dexc in ((1, g.dexca), (0, g.dexcb)):
        if dexc.shape[1] and coeff.size:
            _check(L.orc_apply1(_p(coeff), _p(out), _p(dexc), g.lena, g.lenb,
                                dexc.shape[1], _p(h1c), is_alpha), "apply1")
    return out


def apply_spin1(coeff, h1, g: Graph):
    """sigma for a spin-orbital one-body operator h1 [2n, 2n] (alpha orbitals
    first): the alpha block on alpha strings, the beta block on beta strings
    (fqe_data.py:533-563, lm branch :551-563)."""
    L = lib()
    n = g.norb
    h1 = numpy.asarray(h1, dtype=numpy.complex128)
    coeff = numpy.ascontiguousarray(coeff, dtype=numpy.complex128)
    out = numpy.zeros_like(coeff)
    for is_alpha, dexc, blk in ((1, g.dexca, h1[:n, :n]), (0, g.dexcb, h1[n:, n:])):
        if dexc.shape[1] and coeff.size:
            hb = numpy.ascontiguousarray(blk)
            _check(L.orc_apply1(_p(coeff), _p(out), _p(dexc), g.lena, g.lenb,
                                dexc.shape[1], _p(hb), is_alpha), "apply1 spin")
    return out


def apply_spin12(coeff, h1, h2, g: Graph):
    """sigma for spin-orbital one- and two-body operators h1 [2n, 2n], h2
    [2n]^4 (alpha orbitals first), as _apply_array_spin12_lm
    (fqe_data.py:743-773): the h1'/h2' preparation over all 2n orbitals, the
    same-spin kernel with the alpha-alpha blocks on alpha strings and the
    beta-beta blocks on beta strings, and the opposite-spin kernel with
    h2'[a,a,b,b] + h2'[b,b,a,a] transposed to (k l i j)."""
    L = lib()
    n = g.norb
    h1p, h2p = prep_spatial12(h1, h2)  # the same preparation, over 2n orbitals
    coeff = numpy.ascontiguousarray(coeff, dtype=numpy.complex128)
    out = numpy.zeros_like(coeff)
    if coeff.size == 0 or n == 0:
        return out
    nda = g.dexca.shape[1]
    ndb = g.dexcb.shape[1]
    a, b = slice(0, n), slice(n, 2 * n)
    if nda:
        _check(L.orc_apply12_same_spin(
            _p(coeff), _p(out), _p(g.dexca), g.lena, g.lenb, nda,
            _p(numpy.ascontiguousarray(h1p[a, a])),
            _p(numpy.ascontiguousarray(h2p[a, a, a, a])), n, 1), "spin same alpha")
    if ndb:
        _check(L.orc_apply12_same_spin(
            _p(coeff), _p(out), _p(g.dexcb), g.lena, g.lenb, ndb,
            _p(numpy.ascontiguousarray(h1p[b, b])),
            _p(numpy.ascontiguousarray(h2p[b, b, b, b])), n, 0), "spin same beta")
    if nda and ndb:
        h2ab = numpy.ascontiguousarray(
            h2p[a, a, b, b] + numpy.einsum("ijkl->klij", h2p[b, b, a, a]))
        _check(L.orc_apply12_diff_spin(_p(coeff), _p(out), _p(g.dexca),
                                       _p(g.dexcb), g.lena, g.lenb, nda, ndb,
                                       _p(h2ab), n), "spin diff")
    return out


def compound_matrix(M, strings, norb):
    """C[J][I] = det M[occ(J), occ(I)]: the action of the one-particle map M
    on the determinants of one spin (strings in the graph's order)."""
    occ = [[k for k in range(norb) if (int(s) >> k) & 1] for s in strings]
    n = len(occ)
    C = numpy.ones((n, n), dtype=numpy.complex128)  # no electrons: det of 0x0
    if n and occ[0]:
        for J in range(n):
            for I in range(n):
                C[J, I] = numpy.linalg.det(M[numpy.ix_(occ[J], occ[I])])
    return C


def transform_orbitals(coeff, m_alpha, m_beta, g: Graph):
    """The sector under the orbital maps m_alpha, m_beta [norb, norb]:
    coeff' = C_alpha coeff C_beta^T with C the compound matrices.  The
    reference's Wavefunction.transform (wavefunction.py:813-959) applies
    M = P^T U^H, where P L U = U^H is scipy's LU of the rotation's adjoint,
    through recursive column operators (fqe_data.py:1476-1535)."""
    A = compound_matrix(numpy.asarray(m_alpha), g.astr, g.norb)
    B = compound_matrix(numpy.asarray(m_beta), g.bstr, g.norb)
    return A @ numpy.asarray(coeff, dtype=numpy.complex128) @ B.T


def apply_restricted(coeff, tensors, e_0, g: Graph):
    """One sector of Wavefunction._apply_array (wavefunction.py:366-399):
    apply_inplace by rank, then e_0 * psi if |e_0| > 1e-15."""
    if len(tensors) == 1:
        out = apply_spatial1(coeff, tensors[0], g)
    elif len(tensors) == 2:
        out = apply_spatial12(coeff, tensors[0], tensors[1], g)
    else:
        raise ValueError("oracle covers one- and two-body tensors only")
    if abs(e_0) > 1.0e-15:
        out = out + e_0 * coeff
    return out


def taylor_evolve(coeff, tensors, e_0, time, g: Graph, accuracy=1.0e-15,
                  expansion=30):
    """Taylor propagator (wavefunction.py:553-568, e_0 phase :605-606).
    Returns (result, number of applies)."""
    ham = tuple(-1.0j * time * t for t in tensors)
    result = numpy.array(coeff, dtype=numpy.complex128, copy=True)
    work = numpy.array(coeff, dtype=numpy.complex128, copy=True)
    for order in range(1, expansion):
        work = apply_restricted(work, ham, 0.0, g)
        c = 1.0 / math.factorial(order)
        result += c * work
        if numpy.linalg.norm(work) * abs(c) < accuracy:
            break
    else:
        raise RuntimeError("maximum taylor expansion limit reached")
    if abs(e_0 * time) > 1.0e-15:
        result *= numpy.exp(-1.0j * time * e_0)
    return result, order


def chebyshev_evolve(coeff, tensors, e_0, time, g: Graph, spec_lim,
                     accuracy=1.0e-15, expansion=30):
    """apply_generated_unitary, Chebyshev branch (wavefunction.py:570-602)
    plus the e_0 phase (:605-606), on one sector: with a = (E1 - E0) /
    (2 w'), w' = 0.9875, and shift s = -(E0 + a w'), the series
    exp(-i t (H + s)) = J0(a t) + sum_k 2 (-i)^k J_k(a t) T_k((H + s) / a)
    summed until |T_k psi| |c_k| < accuracy, times exp(i s t) and, for
    e_0 != 0, exp(-i t e_0) (the operator H includes e_0)."""
    from scipy.special import jv
    psi = numpy.asarray(coeff, dtype=numpy.complex128)
    w = 0.9875
    a = (spec_lim[1] - spec_lim[0]) / (2.0 * w)
    shift = -(spec_lim[0] + a * w)

    def h_scaled(v):  # (H + shift) v / a
        return (apply_restricted(v, tensors, e_0, g) + shift * v) / a

    t_prev = psi.copy()
    t_cur = h_scaled(psi)
    out = jv(0, a * time) * psi + 2.0 * jv(1, a * time) * (-1j) * t_cur
    for k in range(2, expansion):
        t_next = 2.0 * h_scaled(t_cur) - t_prev
        t_prev, t_cur = t_cur, t_next
        c = 2.0 * jv(k, a * time) * (-1j) ** k
        out = out + c * t_cur
        if numpy.linalg.norm(t_cur) * abs(c) < accuracy:
            break
    else:
        raise RuntimeError("maximum chebyshev expansion limit reached")
    out = out * numpy.exp(shift * time * 1j)
    if abs(e_0 * time) > 1.0e-15:
        out = out * numpy.exp(-1j * time * e_0)
    return out


def evolve_diagonal_coulomb(coeff, diag, vij, g: Graph):
    """coeff *= exp(E(I)) with diag/vij already holding -i t (fqe_data.py:332-361)."""
    out = numpy.array(coeff, dtype=numpy.complex128, copy=True)
    d = numpy.ascontiguousarray(diag, dtype=numpy.complex128)
    v = numpy.ascontiguousarray(vij, dtype=numpy.complex128)
    if out.size:
        _check(lib().orc_diagonal_coulomb(_p(g.astr), _p(g.bstr), _p(d), _p(v),
                                          _p(out), g.lena, g.lenb, g.norb),
               "diagonal_coulomb")
    return out


def apply_diagonal_coulomb(coeff, diag, vij, g: Graph):
    """coeff *= E(I) (fqe_data.py:263-330)."""
    out = numpy.array(coeff, dtype=numpy.complex128, copy=True)
    d = numpy.ascontiguousarray(diag, dtype=numpy.complex128)
    v = numpy.ascontiguousarray(vij, dtype=numpy.complex128)
    if out.size:
        _check(lib().orc_diagonal_coulomb_apply(_p(g.astr), _p(g.bstr), _p(d),
                                                _p(v), _p(out), g.lena, g.lenb,
                                                g.norb), "dc_apply")
    return out


def make_dvec(coeff, g: Graph):
    """D[i,j] = E_ij coeff, shape [norb, norb, lena, lenb] (fqe_data.py:2209-2234)."""
    norb = g.norb
    coeff = numpy.ascontiguousarray(coeff, dtype=numpy.complex128)
    dvec = numpy.zeros((norb, norb, g.lena, g.lenb), dtype=numpy.complex128)
    L = lib()
    _check(L.orc_make_dvec(_p(g.alens), _p(g.amaps), norb, _p(coeff),
                           _p(dvec), g.lena, g.lenb, 1), "dvec a")
    _check(L.orc_make_dvec(_p(g.blens), _p(g.bmaps), norb, _p(coeff),
                           _p(dvec), g.lena, g.lenb, 0), "dvec b")
    return dvec


def make_coeff(dvec, g: Graph):
    """C_I = sum_ij sum_J <I|E_ij|J> D_ij^J (fqe_data.py:2309-2334)."""
    norb = g.norb
    dvec = numpy.ascontiguousarray(dvec, dtype=numpy.complex128)
    out = numpy.zeros((g.lena, g.lenb), dtype=numpy.complex128)
    L = lib()
    _check(L.orc_make_coeff(_p(g.alens), _p(g.amaps), norb, _p(out), _p(dvec),
                            g.lena, g.lenb, 1), "coeff a")
    _check(L.orc_make_coeff(_p(g.blens), _p(g.bmaps), norb, _p(out), _p(dvec),
                            g.lena, g.lenb, 0), "coeff b")
    return out


def diagonal_energies(h1, h2, g: Graph):
    """<I|H|I> for every determinant by applying H to unit vectors.  O(N)
    applies — this is the reference Davidson's own way of building its
    preconditioner (algorithm/davidson.py:159-180); small cases only."""
    n = g.lena * g.lenb
    out = numpy.zeros(n, dtype=numpy.complex128)
    e = numpy.zeros((g.lena, g.lenb), dtype=numpy.complex128)
    for k in range(n):
        a, b = divmod(k, g.lenb)
        e[a, b] = 1.0
        out[k] = apply_spatial12(e, h1, h2, g)[a, b]
        e[a, b] = 0.0
    return out.reshape(g.lena, g.lenb)


def dense_hamiltonian(h1, h2, g: Graph):
    """Full H matrix by applying H to unit vectors (small cases only)."""
    n = g.lena * g.lenb
    H = numpy.zeros((n, n), dtype=numpy.complex128)
    e = numpy.zeros((g.lena, g.lenb), dtype=numpy.complex128)
    for k in range(n):
        a, b = divmod(k, g.lenb)
        e[a, b] = 1.0
        H[:, k] = apply_spatial12(e, h1, h2, g).ravel()
        e[a, b] = 0.0
    return H


def rdm12(ket, g: Graph, bra=None):
    """FqeData.rdm12(bradata) with ket = self, half-filling form
    (fqe_data.py:1762-1781): with D[i, j, I] = <I|E_ij|.>,
    raw[k, l, i, j] = sum_I conj(D_bra[k, l, I]) D_ket[i, j, I],
    rdm2 = -raw.transpose(1, 2, 0, 3) and rdm2[:, i, i, :] += rdm1; rdm1 as
    rdm1() (= <bra|E_ij|ket>)."""
    bra = ket if bra is None else bra
    dket = make_dvec(ket, g)
    dbra = dket if bra is ket else make_dvec(bra, g)
    r1 = numpy.tensordot(dket, numpy.conj(bra), axes=((2, 3), (0, 1)))
    raw = numpy.tensordot(numpy.conj(dbra), dket, axes=((2, 3), (2, 3)))
    r2 = -raw.transpose(1, 2, 0, 3)
    for i in range(g.norb):
        r2[:, i, i, :] += r1
    return r1, r2


def rdm1(ket, g: Graph, bra=None):
    """FqeData.rdm1(bradata) with ket = self (fqe_data.py:1668-1724):
    rdm1[i][j] = <bra| E_ij |ket> = sum_I conj(bra_I) dvec_ket[i, j, I]."""
    bra = ket if bra is None else bra
    dvec = make_dvec(ket, g)  # [norb, norb, lena, lenb]
    return numpy.tensordot(dvec, numpy.conj(bra), axes=((2, 3), (0, 1)))
