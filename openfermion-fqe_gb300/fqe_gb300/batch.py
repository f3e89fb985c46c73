"""Many sectors' H·psi, or Taylor series, in one CUDA graph (fqegpu_batch_*).

No counterpart in the reference, which applies sectors one at a time
(Wavefunction._apply_array, wavefunction.py:366-399).  A BatchApply takes a
list of FqeData sectors and their operator tuples (as FqeData.apply takes
them), prepares one Hamiltonian handle per sector, runs every apply once
(allocating workspaces and tensor-core plans), records all of them into one
CUDA graph and replays the whole batch with `launch()`.  The graph reads the
coefficient tensors the sectors held at construction (`psis`, kept alive
here); `launch()` refreshes them with `copy_` from a sector whose `coeff`
has since been rebound (FqeData.apply_inplace rebinds it).  Results land in
`sigmas`.
"""

import ctypes
from typing import List, Optional, Sequence

import torch

from . import _lib, settings
from .fqe_data import FqeData, _Ham, _ptr, _stream


class BatchApply:
    def __init__(self, datas: Sequence[FqeData], arrays: Sequence[tuple],
                 alpha: complex = 1.0, beta: complex = 0.0,
                 precision: Optional[str] = None,
                 scratch_limit: Optional[int] = None,
                 autotune: bool = False):
        if len(datas) != len(arrays) or not datas:
            raise ValueError("one operator tuple per sector is required")
        self.datas = list(datas)
        self.hams = []
        for d, arr in zip(self.datas, arrays):
            if not 1 <= len(arr) <= 2:
                raise ValueError("operator tuples hold (h1,) or (h1, h2)")
            ham = _Ham(d._core, arr[0], arr[1] if len(arr) > 1 else None)
            if scratch_limit is not None:
                _lib.call("fqegpu_ham_set_scratch_limit", ham.handle,
                          int(scratch_limit))
            self.hams.append(ham)
        if autotune:
            _tune_all(self.datas, self.hams, precision)
        # the graph records these tensors' addresses: hold them for its life
        self.psis: List[torch.Tensor] = [d.coeff for d in self.datas]
        self.sigmas: List[torch.Tensor] = [torch.empty_like(d.coeff)
                                           for d in self.datas]
        code = (settings.precision_code() if precision is None else
                {"fp64": _lib.PREC_FP64, "ozaki": _lib.PREC_OZAKI}[precision])
        n = len(self.datas)
        hv = (ctypes.c_void_p * n)(*[h.handle.value for h in self.hams])
        pv = (ctypes.c_void_p * n)(*[p.data_ptr() for p in self.psis])
        sv = (ctypes.c_void_p * n)(*[s.data_ptr() for s in self.sigmas])
        a, b = complex(alpha), complex(beta)
        h = ctypes.c_void_p()
        _lib.call("fqegpu_batch_create", n, hv, pv, sv, a.real, a.imag,
                  b.real, b.imag, code, _stream(), ctypes.byref(h))
        self.handle = h

    def launch(self) -> None:
        """Replays the whole batch (asynchronous on the current stream)."""
        for d, p in zip(self.datas, self.psis):
            if d.coeff is not p:
                p.copy_(d.coeff)
        _lib.call("fqegpu_batch_launch", self.handle, _stream())

    def check(self) -> None:
        """Waits for the batch and reports a tensor-core timeout."""
        _lib.call("fqegpu_batch_check", self.handle, _stream())

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.fqegpu_batch_destroy(h)
            self.handle = None


def _tune_all(datas, hams, precision) -> None:
    """The autotuner's choice (fqe_gb300.autotune) for every sector's handle,
    one timing per sector shape."""
    from . import autotune
    prec = precision or ("ozaki" if settings.precision_code() == _lib.PREC_OZAKI
                         else "fp64")
    for d, h in zip(datas, hams):
        autotune.apply_tuning(h, d, prec)


class BatchTaylor:
    """Taylor evolution psi <- exp(-i t H) psi of many sectors in one CUDA
    graph (fqegpu_batch_taylor_create): every sector has its own operator
    tuple (h1, h2) and its own stopping test (||term|| < accuracy, at most
    expansion - 1 orders; Wavefunction.apply_generated_unitary 'taylor',
    wavefunction.py:553-568, sector by sector, without the e_0 phase).  The
    series run on the device as conditional loops in parallel branches of
    one graph; `launch()` evolves every sector's coefficients in place once,
    `terms()` waits and returns the number of terms per sector (RuntimeError
    if a series did not converge).  No counterpart in the reference, which
    evolves one wavefunction at a time."""

    def __init__(self, datas: Sequence[FqeData], arrays: Sequence[tuple],
                 time: float, accuracy: float = 1.0e-15, expansion: int = 30,
                 precision: Optional[str] = None, autotune: bool = False):
        if len(datas) != len(arrays) or not datas:
            raise ValueError("one operator tuple per sector is required")
        self.datas = list(datas)
        self.hams = []
        for d, arr in zip(self.datas, arrays):
            if not 1 <= len(arr) <= 2:
                raise ValueError("operator tuples hold (h1,) or (h1, h2)")
            self.hams.append(_Ham(d._core, arr[0],
                                  arr[1] if len(arr) > 1 else None))
        if autotune:
            _tune_all(self.datas, self.hams, precision)
        # the graph evolves these tensors in place: hold them for its life
        self.psis: List[torch.Tensor] = [d.coeff for d in self.datas]
        code = (settings.precision_code() if precision is None else
                {"fp64": _lib.PREC_FP64, "ozaki": _lib.PREC_OZAKI}[precision])
        n = len(self.datas)
        hv = (ctypes.c_void_p * n)(*[h.handle.value for h in self.hams])
        pv = (ctypes.c_void_p * n)(*[p.data_ptr() for p in self.psis])
        h = ctypes.c_void_p()
        _lib.call("fqegpu_batch_taylor_create", n, hv, pv, float(time),
                  float(accuracy), int(expansion), code, _stream(),
                  ctypes.byref(h))
        self.handle = h

    def launch(self) -> None:
        """One evolution of every sector (asynchronous, in place)."""
        for d, p in zip(self.datas, self.psis):
            if d.coeff is not p:
                p.copy_(d.coeff)
                d.coeff = p
        _lib.call("fqegpu_batch_launch", self.handle, _stream())

    def terms(self) -> List[int]:
        """Waits for the last launch; the number of terms of every series."""
        import numpy
        out = numpy.zeros(len(self.datas), dtype=numpy.int32)
        _lib.call("fqegpu_batch_taylor_terms", self.handle,
                  out.ctypes.data_as(ctypes.c_void_p), _stream())
        return [int(x) for x in out]

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.fqegpu_batch_destroy(h)
            self.handle = None
