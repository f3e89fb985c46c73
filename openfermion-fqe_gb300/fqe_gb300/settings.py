"""Global settings (the analogue of fqe/settings.py).

``precision`` selects the contraction arithmetic of every apply and Taylor
step: "fp64" is the plain FP64 path that reproduces the reference to rounding;
"ozaki" runs the pair contraction on the tcgen05 tensor cores with FP64
operands split into BF16 slices (real integrals; complex tensors fall back to
the FP64 kernel on the GPU).  The reference's own switch between its C and
Python code paths is ``fqe.settings.use_accelerated_code`` (settings.py:37).
"""

import torch

from . import _lib

precision = "fp64"

global_max_norb = 64
"""The global maximum number of orbitals (settings.py:40)."""

_device_index = 0


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("fqe_gb300 requires a CUDA device; there is no CPU "
                           "path")
    return torch.device("cuda", _device_index)


def precision_code() -> int:
    if precision == "fp64":
        return _lib.PREC_FP64
    if precision == "ozaki":
        return _lib.PREC_OZAKI
    raise ValueError(f"unknown precision {precision!r}")
