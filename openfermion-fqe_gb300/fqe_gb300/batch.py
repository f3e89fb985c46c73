"""Many sectors' H·psi in one CUDA graph (fqegpu_batch_*).

No counterpart in the reference, which applies sectors one at a time
(Wavefunction._apply_array, wavefunction.py:366-399).  A BatchApply takes a
list of FqeData sectors and their operator tuples (as FqeData.apply takes
them), prepares one Hamiltonian handle per sector, runs every apply once
(allocating workspaces and tensor-core plans), records all of them into one
CUDA graph and replays the whole batch with `launch()`.  Inputs are the
sectors' own coefficient tensors; results land in `sigmas`.
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
                 scratch_limit: Optional[int] = None):
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
        self.sigmas: List[torch.Tensor] = [torch.empty_like(d.coeff)
                                           for d in self.datas]
        code = (settings.precision_code() if precision is None else
                {"fp64": _lib.PREC_FP64, "ozaki": _lib.PREC_OZAKI}[precision])
        n = len(self.datas)
        hv = (ctypes.c_void_p * n)(*[h.handle.value for h in self.hams])
        pv = (ctypes.c_void_p * n)(*[d.coeff.data_ptr() for d in self.datas])
        sv = (ctypes.c_void_p * n)(*[s.data_ptr() for s in self.sigmas])
        a, b = complex(alpha), complex(beta)
        h = ctypes.c_void_p()
        _lib.call("fqegpu_batch_create", n, hv, pv, sv, a.real, a.imag,
                  b.real, b.imag, code, _stream(), ctypes.byref(h))
        self.handle = h

    def launch(self) -> None:
        """Replays the whole batch (asynchronous on the current stream)."""
        _lib.call("fqegpu_batch_launch", self.handle, _stream())

    def check(self) -> None:
        """Waits for the batch and reports a tensor-core timeout."""
        _lib.call("fqegpu_batch_check", self.handle, _stream())

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.fqegpu_batch_destroy(h)
            self.handle = None
