"""FqeData: the coefficients of one (nalpha, nbeta) sector, resident on the GPU.

Mirrors ``fqe.fqe_data.FqeData`` (fqe_data.py:61-3076) on the H·psi path:
construction, ``apply`` / ``apply_inplace`` for one- and two-body spatial
tensors, the diagonal-Coulomb apply and evolve, the dvec gather/scatter and
the vector operations.  ``coeff`` is a ``torch.complex128`` CUDA tensor of
shape [lena, lenb], alpha-major, the layout of the reference's numpy array.
Every operation runs in libfqegpu.so; there is no CPU path.
"""

import copy
import ctypes
import hashlib
from collections import OrderedDict
from typing import Optional, Tuple

import numpy
import torch

from . import _lib
from . import settings
from .fci_graph import FciGraph, get_graph


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


def _host_c128(a) -> numpy.ndarray:
    return numpy.ascontiguousarray(a, dtype=numpy.complex128)


class _Ham:
    """Owner of one fqegpu_ham handle: a restricted operator (h1 [n, n],
    h2 [n]^4) or, with spin=True, a spin-orbital one (h1 [2n, 2n], h2
    [2n]^4, alpha orbitals first)."""

    def __init__(self, graph: FciGraph, h1, h2, spin: bool = False):
        self.graph = graph  # keeps the graph alive as long as the handle
        self.spin = spin
        self._h1 = None if h1 is None else _host_c128(h1)
        self._h2 = None if h2 is None else _host_c128(h2)
        h = ctypes.c_void_p()
        _lib.call(
            "fqegpu_ham_create_spin" if spin else "fqegpu_ham_create", graph.handle,
            None if self._h1 is None else self._h1.ctypes.data_as(
                ctypes.c_void_p),
            None if self._h2 is None else self._h2.ctypes.data_as(
                ctypes.c_void_p), None, ctypes.byref(h))
        self.handle = h
        info = numpy.zeros(4, dtype=numpy.int64)
        _lib.call("fqegpu_ham_info", h, info.ctypes.data_as(ctypes.c_void_p))
        self.npairs, self.compressed, self.real = (int(info[0]),
                                                   bool(info[1]),
                                                   bool(info[2]))

    def __del__(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            try:
                _lib.load().fqegpu_ham_destroy(self.handle)
            except Exception:
                pass
            self.handle = None


_HAM_CACHE: "OrderedDict[tuple, _Ham]" = OrderedDict()
_HAM_CACHE_SIZE = 8


def _digest(a) -> Optional[bytes]:
    if a is None:
        return None
    a = _host_c128(a)
    return hashlib.blake2b(a.tobytes(), digest_size=16).digest() + bytes(
        str(a.shape), "ascii")


def ham_for(graph: FciGraph, h1, h2, spin: bool = False) -> _Ham:
    """Prepared Hamiltonian for a sector, cached on the tensors' contents."""
    key = (graph.nalpha(), graph.nbeta(), graph.norb(), spin, _digest(h1),
           _digest(h2))
    ham = _HAM_CACHE.get(key)
    if ham is None:
        ham = _Ham(graph, h1, h2, spin)
        _HAM_CACHE[key] = ham
        while len(_HAM_CACHE) > _HAM_CACHE_SIZE:
            _HAM_CACHE.popitem(last=False)
    else:
        _HAM_CACHE.move_to_end(key)
    return ham


def clear_ham_cache() -> None:
    """Drops the cached Hamiltonian handles (their device workspaces are
    freed once nothing else holds them)."""
    _HAM_CACHE.clear()


def check_apply(ham: "_Ham") -> None:
    """Waits for the current stream and raises TimeoutError if a tensor-core
    apply of `ham` gave up a bounded device wait since the last check."""
    _lib.call("fqegpu_ham_check", ham.handle, _stream())


def rdm2_from_gram(raw: numpy.ndarray, rdm1: numpy.ndarray) -> numpy.ndarray:
    """rdm2 of FqeData.rdm12 (fqe_data.py:1762-1781) from the Gram matrix
    raw[kl][ij] = sum_I conj(D_bra[kl, I]) D_ket[ij, I] of the dvecs and
    rdm1[i][j] = <bra|E_ij|ket>: rdm2 = -raw.reshape(n,n,n,n) permuted to
    (l, i, k, j) order, i.e. rdm2[a, b, c, d] = -raw[c, a, b, d], and
    rdm2[:, i, i, :] += rdm1."""
    norb = rdm1.shape[0]
    r2 = -numpy.ascontiguousarray(
        raw.reshape(norb, norb, norb, norb).transpose(1, 2, 0, 3))
    for i in range(norb):
        r2[:, i, i, :] += rdm1
    return r2


class FqeData:
    """One (nalpha, nbeta, norb) sector."""

    def __init__(self,
                 nalpha: int,
                 nbeta: int,
                 norb: int,
                 fcigraph: Optional[FciGraph] = None,
                 dtype=numpy.complex128) -> None:
        if fcigraph is not None and (nalpha != fcigraph.nalpha() or
                                     nbeta != fcigraph.nbeta() or
                                     norb != fcigraph.norb()):
            raise ValueError("FciGraph does not match other parameters")
        if dtype not in (numpy.complex128, complex):
            raise TypeError("only complex128 coefficients are supported")
        self._core = fcigraph if fcigraph is not None else get_graph(
            nalpha, nbeta, norb)
        self._dtype = numpy.complex128
        self._nele = nalpha + nbeta
        self._m_s = nalpha - nbeta
        self.coeff = torch.zeros((self._core.lena(), self._core.lenb()),
                                 dtype=torch.complex128,
                                 device=settings.device())

    # -- accessors -------------------------------------------------------
    def lena(self) -> int:
        return self._core.lena()

    def lenb(self) -> int:
        return self._core.lenb()

    def nalpha(self) -> int:
        return self._core.nalpha()

    def nbeta(self) -> int:
        return self._core.nbeta()

    def norb(self) -> int:
        return self._core.norb()

    def n_electrons(self) -> int:
        return self._nele

    def __hash__(self):
        return hash((self._nele, self._m_s))

    def __getitem__(self, key: Tuple[int, int]) -> complex:
        a = self._core.index_alpha(key[0])
        b = self._core.index_beta(key[1])
        return complex(self.coeff[a, b].item())

    def __setitem__(self, key: Tuple[int, int], value: complex) -> None:
        a = self._core.index_alpha(key[0])
        b = self._core.index_beta(key[1])
        self.coeff[a, b] = value

    def alpha_map(self, iorb: int, jorb: int):
        return self._core.alpha_map(iorb, jorb)

    def beta_map(self, iorb: int, jorb: int):
        return self._core.beta_map(iorb, jorb)

    def get_fcigraph(self) -> FciGraph:
        return self._core

    def to_numpy(self) -> "numpy.ndarray":
        return self.coeff.detach().cpu().numpy()

    # -- set-up ------------------------------------------------------------
    def set_wfn(self, strategy: str = "ones", raw_data=None) -> None:
        """fqe_data.py set_wfn: 'ones', 'zero', 'random' or 'from_data'."""
        shape = (self.lena(), self.lenb())
        if strategy == "ones":
            self.coeff.fill_(1.0 + 0.0j)
        elif strategy == "zero":
            self.coeff.zero_()
        elif strategy == "random":
            rng = numpy.random.default_rng()
            data = rng.standard_normal(shape) + 1.0j * rng.standard_normal(
                shape)
            self.coeff.copy_(torch.from_numpy(data))
        elif strategy == "from_data":
            data = raw_data
            if isinstance(data, torch.Tensor):
                if tuple(data.shape) != shape:
                    raise ValueError("raw_data has the wrong shape")
                self.coeff.copy_(data.to(torch.complex128))
            else:
                data = _host_c128(data)
                if data.shape != shape:
                    raise ValueError("raw_data has the wrong shape")
                self.coeff.copy_(torch.from_numpy(data))
        else:
            raise ValueError(f"Unknown option for strategy: {strategy}")

    # -- vector operations (fqe_data.py:2620-2751) ---------------------------
    def ax_plus_y(self, sval: complex, other: "FqeData") -> "FqeData":
        assert hash(self) == hash(other)
        s = complex(sval)
        _lib.call("fqegpu_axpy", self.coeff.numel(), s.real, s.imag,
                  _ptr(other.coeff), _ptr(self.coeff), _stream())
        return self

    def scale(self, sval: complex) -> None:
        s = complex(sval)
        _lib.call("fqegpu_scale", self.coeff.numel(), s.real, s.imag,
                  _ptr(self.coeff), _stream())

    def norm(self) -> float:
        out = ctypes.c_double()
        _lib.call("fqegpu_norm2", self.coeff.numel(), _ptr(self.coeff),
                  ctypes.byref(out), _stream())
        return out.value

    def vdot(self, other: "FqeData") -> complex:
        """sum conj(self) * other."""
        out = (ctypes.c_double * 2)()
        _lib.call("fqegpu_vdot", self.coeff.numel(), _ptr(self.coeff),
                  _ptr(other.coeff), out, _stream())
        return complex(out[0], out[1])

    def fill(self, value: complex) -> None:
        self.coeff.fill_(complex(value))

    def conj(self) -> None:
        self.coeff.copy_(torch.conj_physical(self.coeff))

    # -- H·psi (fqe_data.py:404-531, 582-710) --------------------------------
    def apply(self, array: Tuple[numpy.ndarray, ...]) -> "FqeData":
        out = copy.deepcopy(self)
        out.apply_inplace(array)
        return out

    def apply_inplace(self, array: Tuple[numpy.ndarray, ...]) -> None:
        len_arr = len(array)
        if len_arr < 1 or len_arr > 4:
            raise ValueError("Number of operators in tuple must be "
                             "between 1 and 4.")
        first = next((x for x in array if isinstance(x, numpy.ndarray)), None)
        if first is None:
            return
        spatial = first.shape[0] == self.norb()
        if not spatial and first.shape[0] != 2 * self.norb():
            raise ValueError("Inconsistent number of spin-orbitals in "
                             "operators and wavefunction.")
        if len_arr > 2:
            raise NotImplementedError(
                "only one- and two-body operators are on this path")
        if spatial:
            if len_arr == 1:
                self.coeff = self._apply_array_spatial1(array[0])
            else:
                self.coeff = self._apply_array_spatial12(array[0], array[1])
        elif len_arr == 1:
            self.coeff = self._apply_array_spin1(array[0])
        else:
            self.coeff = self._apply_array_spin12(array[0], array[1])

    def _run_apply(self, ham: _Ham, alpha=1.0, beta=0.0,
                   out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """alpha H coeff + beta coeff, asynchronous on the current stream (a
        tensor-core timeout is reported by check_apply or the handle's next
        apply)."""
        if out is None:
            out = torch.empty_like(self.coeff)
        a, b = complex(alpha), complex(beta)
        _lib.call("fqegpu_apply", ham.handle, _ptr(self.coeff), _ptr(out),
                  a.real, a.imag, b.real, b.imag, settings.precision_code(),
                  _stream())
        return out

    def _apply_array_spatial1(self, h1e: numpy.ndarray) -> torch.Tensor:
        norb = self.norb()
        assert h1e.shape == (norb, norb)
        return self._run_apply(ham_for(self._core, h1e, None))

    def _apply_array_spatial12(self, h1e: numpy.ndarray,
                               h2e: numpy.ndarray) -> torch.Tensor:
        norb = self.norb()
        assert h1e.shape == (norb, norb)
        assert h2e.shape == (norb, norb, norb, norb)
        return self._run_apply(ham_for(self._core, h1e, h2e))

    def _apply_array_spin1(self, h1e: numpy.ndarray) -> torch.Tensor:
        """fqe_data.py:533-563: the alpha block of h1e on alpha strings, the
        beta block on beta strings (fqegpu_ham_create_spin, one-body)."""
        norb = self.norb()
        assert h1e.shape == (norb * 2, norb * 2)
        return self._run_apply(ham_for(self._core, h1e, None, spin=True))

    def _apply_array_spin12(self, h1e: numpy.ndarray,
                            h2e: numpy.ndarray) -> torch.Tensor:
        """fqe_data.py:614-635, 743-773: spin-orbital one- and two-body
        operators (fqegpu_ham_create_spin)."""
        norb = self.norb()
        assert h1e.shape == (norb * 2, norb * 2)
        assert h2e.shape == (norb * 2, norb * 2, norb * 2, norb * 2)
        return self._run_apply(ham_for(self._core, h1e, h2e, spin=True))

    # -- orbital rotation and diagonal evolution ------------------------------
    def apply_columns_recursive_inplace(self, mat1: numpy.ndarray,
                                        mat2: numpy.ndarray) -> None:
        """fqe_data.py:1510-1535: for every column icol, first of the alpha
        strings with mat1 and then of the beta strings with mat2, the
        column operator 1 + sum_i mat[i, icol] E_{i,icol}, applied in order
        (fqegpu_transform; the work array is temporary device memory)."""
        m1 = _host_c128(mat1)
        m2 = _host_c128(mat2)
        work = torch.empty_like(self.coeff)
        _lib.call("fqegpu_transform", self._core.handle,
                  m1.ctypes.data_as(ctypes.c_void_p),
                  m2.ctypes.data_as(ctypes.c_void_p), _ptr(self.coeff),
                  _ptr(work), _stream())

    def evolve_diagonal(self, array: numpy.ndarray,
                        inplace: bool = False) -> torch.Tensor:
        """fqe_data.py:203-262: coeff[a, b] *= exp(sum_{i in a} array[i] +
        sum_{j in b} array[beta_ptr + j]), array of size norb or 2 norb."""
        norb = self.norb()
        array = _host_c128(array).reshape(-1)
        if array.size == 2 * norb:
            da, db = array[:norb].copy(), array[norb:].copy()
        elif array.size == norb:
            da, db = array, array
        else:
            raise ValueError('Non-diagonal array passed into evolve_diagonal')
        data = self.coeff if inplace else self.coeff.clone()
        _lib.call("fqegpu_evolve_diagonal", self._core.handle,
                  da.ctypes.data_as(ctypes.c_void_p),
                  db.ctypes.data_as(ctypes.c_void_p), _ptr(data), _stream())
        return data

    # -- diagonal Coulomb (fqe_data.py:263-402) ------------------------------
    def _diag_coulomb(self, diag, array, inplace: bool, mode: int):
        data = self.coeff if inplace else self.coeff.clone()
        d = _host_c128(diag)
        v = _host_c128(array)
        _lib.call("fqegpu_diagonal_coulomb", self._core.handle,
                  d.ctypes.data_as(ctypes.c_void_p),
                  v.ctypes.data_as(ctypes.c_void_p), _ptr(data), mode,
                  _stream())
        return data

    def apply_diagonal_coulomb(self, diag, array,
                               inplace: bool = False) -> torch.Tensor:
        return self._diag_coulomb(diag, array, inplace, 1)

    def evolve_diagonal_coulomb(self, diag, array,
                                inplace: bool = False) -> torch.Tensor:
        return self._diag_coulomb(diag, array, inplace, 0)

    # -- dvec (fqe_data.py:2149-2234, 2309-2334) -----------------------------
    def calculate_dvec_spatial(self) -> torch.Tensor:
        norb = self.norb()
        dvec = torch.empty((norb, norb, self.lena(), self.lenb()),
                           dtype=torch.complex128, device=self.coeff.device)
        if dvec.numel():
            _lib.call("fqegpu_make_dvec", self._core.handle, _ptr(self.coeff),
                      _ptr(dvec), _stream())
        return dvec

    def _calculate_coeff_spatial_with_dvec(self,
                                           dvec: torch.Tensor) -> torch.Tensor:
        dvec = dvec.contiguous()
        out = torch.zeros_like(self.coeff)
        if dvec.numel():
            _lib.call("fqegpu_make_coeff", self._core.handle, _ptr(dvec),
                      _ptr(out), 0, _stream())
        return out

    # -- Davidson support -----------------------------------------------------
    def rdm1(self, bradata: Optional["FqeData"] = None):
        """fqe_data.py:1668-1724: (rdm1,) with rdm1[i][j] = <bra| E_ij |self>,
        bra = bradata or self (spin-summed, complex128 [norb][norb])."""
        bra = self if bradata is None else bradata
        if (bra.nalpha(), bra.nbeta(), bra.norb()) != (
                self.nalpha(), self.nbeta(), self.norb()):
            raise ValueError("rdm1: bra and ket sectors differ")
        norb = self.norb()
        out = numpy.zeros((norb, norb), dtype=numpy.complex128)
        _lib.call("fqegpu_rdm1", self._core.handle, _ptr(bra.coeff),
                  _ptr(self.coeff), out.ctypes.data_as(ctypes.c_void_p),
                  _stream())
        return (out,)

    def rdm12(self, bradata: Optional["FqeData"] = None):
        """fqe_data.py:1726-1838 in its half-filling form (the branches of the
        reference that honour the bra agree with it): (rdm1, rdm2) with
        rdm1[i][j] = <bra| E_ij |self> and
        rdm2[a][b][c][d] = <bra| sum_st a+_as a+_bt a_cs a_dt |self>.
        The Gram matrix of the two dvecs comes from fqegpu_rdm2_gram, which
        forms the dvecs on the fly (no norb^2-times-sector array)."""
        bra = self if bradata is None else bradata
        if (bra.nalpha(), bra.nbeta(), bra.norb()) != (
                self.nalpha(), self.nbeta(), self.norb()):
            raise ValueError("rdm12: bra and ket sectors differ")
        r1 = self.rdm1(bradata)[0]
        norb = self.norb()
        raw = numpy.zeros((norb * norb, norb * norb), dtype=numpy.complex128)
        if raw.size:
            _lib.call("fqegpu_rdm2_gram", self._core.handle, _ptr(bra.coeff),
                      _ptr(self.coeff), raw.ctypes.data_as(ctypes.c_void_p),
                      _stream())
        return r1, rdm2_from_gram(raw, r1)

    def diagonal_energies(self, h1e, h2e) -> torch.Tensor:
        """<I|H|I> for every determinant (Slater-Condon, one pass)."""
        ham = ham_for(self._core, h1e, h2e)
        out = torch.empty((self.lena(), self.lenb()), dtype=torch.float64,
                          device=self.coeff.device)
        _lib.call("fqegpu_diagonal", ham.handle, _ptr(out), _stream())
        return out

    # pickling (Wavefunction.save / read): the sector and the coefficients as
    # a host array; the string graph is rebuilt on the device when loaded
    def __getstate__(self):
        return {"nalpha": self.nalpha(), "nbeta": self.nbeta(),
                "norb": self.norb(), "coeff": self.to_numpy()}

    def __setstate__(self, state):
        self._core = get_graph(state["nalpha"], state["nbeta"], state["norb"])
        self._dtype = numpy.complex128
        self._nele = state["nalpha"] + state["nbeta"]
        self._m_s = state["nalpha"] - state["nbeta"]
        self.coeff = torch.from_numpy(
            numpy.ascontiguousarray(state["coeff"], dtype=numpy.complex128)).to(
                settings.device())

    def __deepcopy__(self, memo):
        new = FqeData.__new__(FqeData)
        new._core = self._core
        new._dtype = self._dtype
        new._nele = self._nele
        new._m_s = self._m_s
        new.coeff = self.coeff.clone()
        return new
