"""Autotuner of the apply's launch shape per sector shape.

No counterpart in the reference, whose applies are CPU loops without
tunables.  For a sector shape (norb, nalpha, nbeta) and the tensor-core
precision it times fqegpu_apply (CUDA events on the current stream, after a
warm-up) over the candidates

* tiles of 32 determinants per column super-block of the tile order (alpha
  rows run inside a super-block, so the super-block's rows of psi's digit
  planes stay in L2 while every alpha row's gathers read them): 8, 16, 32, 64;
* for sectors of at most 65,536 determinants, the FP64 kernels instead of the
  tensor-core form (never less accurate; their fixed costs are lower)

and keeps the fastest (fqegpu_ham_set_tuning).  Choices are cached per
(shape, pair count, precision), so one timing serves every handle of that
shape (the many sectors of a batch).
"""

from typing import Dict, Optional, Tuple

import torch

from . import _lib
from .fqe_data import FqeData, _Ham

SUPER_TILES = (8, 16, 32, 64)
DEFAULT = {"super_tiles": 32, "fp64": False}
SMALL_SECTOR = 65536

_cache: Dict[Tuple, dict] = {}


def _key(data: FqeData, ham: _Ham, precision: str) -> Tuple:
    return (data.norb(), data.nalpha(), data.nbeta(), ham.npairs, ham.compressed,
            ham.real, precision)


def set_tuning(ham: _Ham, choice: dict) -> None:
    _lib.call("fqegpu_ham_set_tuning", ham.handle, int(choice["super_tiles"]),
              1 if choice["fp64"] else 0)


def _time(ham: _Ham, data: FqeData, out: torch.Tensor, reps: int) -> float:
    from .fqe_data import _ptr, _stream
    stream = torch.cuda.current_stream()

    def run():
        _lib.call("fqegpu_apply", ham.handle, _ptr(data.coeff), _ptr(out), 1.0,
                  0.0, 0.0, 0.0, _lib.PREC_OZAKI, _stream())
    run()  # warm-up (and the workspace of the candidate)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    e1.synchronize()
    _lib.call("fqegpu_ham_check", ham.handle, _stream())
    return e0.elapsed_time(e1) / reps


def tune(ham: _Ham, data: FqeData, reps: int = 3,
         precision: str = "ozaki") -> dict:
    """Times the candidates on this handle and sector, applies and caches
    the fastest; returns it with the timings ({"super_tiles", "fp64",
    "ms", "timings"})."""
    if precision != "ozaki":
        return dict(DEFAULT, ms=None, timings={})
    out = torch.empty_like(data.coeff)
    timings = {}
    for st in SUPER_TILES:
        c = {"super_tiles": st, "fp64": False}
        set_tuning(ham, c)
        timings[f"tensor/super{st}"] = (_time(ham, data, out, reps), c)
    if data.lena() * data.lenb() <= SMALL_SECTOR:
        c = {"super_tiles": 32, "fp64": True}
        set_tuning(ham, c)
        timings["fp64"] = (_time(ham, data, out, reps), c)
    name = min(timings, key=lambda k: timings[k][0])
    best = dict(timings[name][1])
    set_tuning(ham, best)
    best["ms"] = timings[name][0]
    best["timings"] = {k: v[0] for k, v in timings.items()}
    _cache[_key(data, ham, precision)] = best
    return best


def apply_tuning(ham: _Ham, data: FqeData, precision: str = "ozaki",
                 reps: int = 3) -> dict:
    """The cached choice for this shape (tuned on first use), applied to
    `ham`."""
    k = _key(data, ham, precision)
    if k not in _cache:
        return tune(ham, data, reps, precision)
    set_tuning(ham, _cache[k])
    return _cache[k]


def cached() -> Dict[Tuple, dict]:
    return dict(_cache)


def clear() -> None:
    _cache.clear()
