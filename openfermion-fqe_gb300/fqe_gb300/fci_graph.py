"""FciGraph: the string addressing of one (nalpha, nbeta, norb) sector.

Mirrors ``fqe.fci_graph.FciGraph`` (fci_graph.py:99-570): same constructor
checks and messages, same accessors.  The tables are built on the GPU by
``fqegpu_graph_create`` (K1) and stay there; the reference-format views
(``_astr``, ``_alpha_map``, ``_dexca`` ...) are copied out lazily for callers
and tests that want them on the host.
"""

import ctypes
from typing import Dict, List, Tuple

import numpy

from . import _lib


class FciGraph:
    """Knowles-Handy addressing of determinants {alpha}{beta}|0>."""

    def __init__(self, nalpha: int, nbeta: int, norb: int) -> None:
        # same checks and messages as fci_graph.py:124-137
        if norb < 0:
            raise ValueError(f'norb needs to be >= 0, passed value is {norb}')
        if nalpha < 0:
            raise ValueError(
                f'nalpha needs to be >= 0, passed value is {nalpha}')
        if nbeta < 0:
            raise ValueError(f'nbeta needs to be >= 0, passed value is {nbeta}')
        if nalpha > norb:
            raise ValueError(
                f'nalpha needs to be <= norb, passed value is {nbeta}')
        if nbeta > norb:
            raise ValueError(
                f'nbeta needs to be <= norb, passed value is {nbeta}')
        self._norb = norb
        self._nalpha = nalpha
        self._nbeta = nbeta
        handle = ctypes.c_void_p()
        _lib.call("fqegpu_graph_create", norb, nalpha, nbeta, None,
                  ctypes.byref(handle))
        self._handle = handle
        lena, lenb = ctypes.c_int64(), ctypes.c_int64()
        nda, ndb = ctypes.c_int(), ctypes.c_int()
        _lib.call("fqegpu_graph_dims", handle, ctypes.byref(lena),
                  ctypes.byref(lenb), ctypes.byref(nda), ctypes.byref(ndb))
        self._lena, self._lenb = lena.value, lenb.value
        self._ndexca, self._ndexcb = nda.value, ndb.value
        self._host: Dict[str, object] = {}

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                _lib.load().fqegpu_graph_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._handle = None

    @property
    def handle(self):
        return self._handle

    # -- sizes --------------------------------------------------------------
    def lena(self) -> int:
        return self._lena

    def lenb(self) -> int:
        return self._lenb

    def nalpha(self) -> int:
        return self._nalpha

    def nbeta(self) -> int:
        return self._nbeta

    def norb(self) -> int:
        return self._norb

    # -- host copies of the device tables -----------------------------------
    def _strings(self, spin: int) -> numpy.ndarray:
        key = f"str{spin}"
        if key not in self._host:
            n = self._lena if spin == 0 else self._lenb
            out = numpy.zeros(n, dtype=numpy.uint64)
            _lib.call("fqegpu_graph_strings", self._handle, spin,
                      out.ctypes.data_as(ctypes.c_void_p))
            self._host[key] = out
        return self._host[key]

    def _dexc(self, spin: int) -> numpy.ndarray:
        key = f"dexc{spin}"
        if key not in self._host:
            n = self._lena if spin == 0 else self._lenb
            nd = self._ndexca if spin == 0 else self._ndexcb
            out = numpy.zeros((n, nd, 3), dtype=numpy.int32)
            if out.size:
                _lib.call("fqegpu_graph_dexc", self._handle, spin,
                          out.ctypes.data_as(ctypes.c_void_p))
            self._host[key] = out
        return self._host[key]

    def _maps(self, spin: int) -> Dict[Tuple[int, int], numpy.ndarray]:
        key = f"maps{spin}"
        if key not in self._host:
            norb = self._norb
            lens = numpy.zeros((norb, norb), dtype=numpy.int32)
            if norb:
                _lib.call("fqegpu_graph_map_lengths", self._handle, spin,
                          lens.ctypes.data_as(ctypes.c_void_p))
            flat = numpy.zeros((max(int(lens.sum()), 1), 3), dtype=numpy.int32)
            if lens.sum():
                _lib.call("fqegpu_graph_maps", self._handle, spin,
                          flat.ctypes.data_as(ctypes.c_void_p))
            out = {}
            off = 0
            for i in range(norb):
                for j in range(norb):
                    n = int(lens[i, j])
                    out[(i, j)] = flat[off:off + n].copy()
                    off += n
            self._host[key] = out
        return self._host[key]

    def _zmatrix(self, spin: int) -> numpy.ndarray:
        nele = self._nalpha if spin == 0 else self._nbeta
        out = numpy.zeros((nele, self._norb), dtype=numpy.int32)
        if out.size:
            _lib.call("fqegpu_graph_zmatrix", self._handle, spin,
                      out.ctypes.data_as(ctypes.c_void_p))
        return out

    @property
    def _astr(self) -> numpy.ndarray:
        return self._strings(0)

    @property
    def _bstr(self) -> numpy.ndarray:
        return self._strings(1)

    @property
    def _dexca(self) -> numpy.ndarray:
        return self._dexc(0)

    @property
    def _dexcb(self) -> numpy.ndarray:
        return self._dexc(1)

    @property
    def _alpha_map(self) -> Dict[Tuple[int, int], numpy.ndarray]:
        return self._maps(0)

    @property
    def _beta_map(self) -> Dict[Tuple[int, int], numpy.ndarray]:
        return self._maps(1)

    @property
    def _aind(self) -> Dict[int, int]:
        return {int(s): k for k, s in enumerate(self._astr)}

    @property
    def _bind(self) -> Dict[int, int]:
        return {int(s): k for k, s in enumerate(self._bstr)}

    def alpha_map(self, iorb: int, jorb: int) -> numpy.ndarray:
        return self._alpha_map[(iorb, jorb)]

    def beta_map(self, iorb: int, jorb: int) -> numpy.ndarray:
        return self._beta_map[(iorb, jorb)]

    def string_alpha(self, address: int) -> int:
        return int(self._astr[address])

    def string_beta(self, address: int) -> int:
        return int(self._bstr[address])

    def string_alpha_all(self) -> numpy.ndarray:
        return self._astr

    def string_beta_all(self) -> numpy.ndarray:
        return self._bstr

    def index_alpha(self, bit_string: int) -> int:
        return self._aind[int(bit_string)]

    def index_beta(self, bit_string: int) -> int:
        return self._bind[int(bit_string)]

    def z_matrix(self, spin: int = 0) -> numpy.ndarray:
        return self._zmatrix(spin)

    def __repr__(self) -> str:
        return (f"FciGraph(nalpha={self._nalpha}, nbeta={self._nbeta}, "
                f"norb={self._norb})")


_GRAPHS: Dict[Tuple[int, int, int], FciGraph] = {}


def get_graph(nalpha: int, nbeta: int, norb: int) -> FciGraph:
    """Shared graph per sector shape (the tables are read-only)."""
    key = (nalpha, nbeta, norb)
    g = _GRAPHS.get(key)
    if g is None:
        g = FciGraph(nalpha, nbeta, norb)
        _GRAPHS[key] = g
    return g


def alpha_beta_strings(graph: FciGraph) -> List[numpy.ndarray]:
    return [graph._astr, graph._bstr]
